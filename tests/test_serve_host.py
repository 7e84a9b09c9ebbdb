"""Host side of the request loop: the admission footprint estimate (no GPU needed)."""
import ctypes as C

from metapart_gb300 import serve, synth


def _fp(data: bytes, k=31, scans=1, threads=2, chunks=4, min3=0, il=0):
    buf = C.create_string_buffer(data, len(data))
    return serve.footprint(C.addressof(buf), len(data), serve.RequestParams(k, min3, scans, threads, chunks, il))


def test_footprint_covers_input_output_and_tuples(built_gpu):
    small = synth.fastq_bytes(synth.workload("plain_small", 5000, seed=1))
    large = synth.fastq_bytes(synth.workload("plain_small", 50000, seed=1))
    fs, fl = _fp(small), _fp(large)
    assert fl > fs > 0
    # FASTQ in and out, and two 13-byte tuple buffers for (nearly) every base of the one scan
    bases = 50000 * 100
    assert fl >= 2 * len(large) + 26 * bases
    assert _fp(large, scans=2) < fl            # a second scan halves the largest tuple buffers
    assert _fp(large, il=1) > fl               # interleaved output may hold each pair twice
    assert fl < 64 * len(large) + (256 << 20)  # and the estimate stays proportionate
    # the count pass's store of the reads: 9 bytes per position for the k-mer cache, 0.375 per base packed
    buf = C.create_string_buffer(large, len(large))
    fp = {st: serve.footprint(C.addressof(buf), len(large), serve.RequestParams(31, 0, 1, 2, 4, 0, st))
          for st in (0, 1, 2)}
    assert fp[0] < fp[2] < fp[1]
    assert fp[1] - fp[0] >= 9 * bases and fp[2] - fp[0] < bases
