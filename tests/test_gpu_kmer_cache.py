"""The count pass's stores of the reads: a job that counts and partitions in one go with the k-mer cache
(the default) or with the 2-bit packed reads gives every stage dump, label and partition file byte-identical
to the same job with no store (k-mers recomputed from the FASTQ bytes, the path the drop-in programs take and
the parity tests pin to the oracle).  A read with a byte the packed reads cannot hold makes the job fall back
to the FASTQ bytes, with the same results; the overlapped load-and-count call keeps the packed reads in
pieces, one per upload segment."""
import numpy as np
import pytest

from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu

CASES = [
    ("plain_small", 20000, 27, 4, 1, 2, False),
    ("plain_large", 30000, 31, 8, 2, 4, False),
    ("plain_small", 12000, 25, 6, 3, 3, False),
    ("hotspot", 30000, 31, 4, 1, 2, False),
    ("interleaved_small", 20000, 27, 4, 2, 2, True),
    ("plain_small", 8000, 11, 4, 2, 2, False),
]


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


def _run(ctx, data, k, chunks, scans, threads, il, store, d):
    d.mkdir()
    job, bounds, _ = native.run_pipeline(ctx, data, k, chunks, scans, threads, interleaved=il, dump_dir=str(d),
                                         store=store)
    try:
        out, sizes = job.output()
        return bytes(out), sizes.copy(), bounds.copy(), job.labels()
    finally:
        job.close()


@pytest.mark.parametrize("store", ["kmer_cache", "packed"])
@pytest.mark.parametrize("name,n,k,chunks,scans,threads,il", CASES,
                         ids=[f"{c[0]}-k{c[2]}-s{c[4]}" for c in CASES])
def test_store_matches_recomputed(ctx, tmp_path, name, n, k, chunks, scans, threads, il, store):
    data = synth.fastq_bytes(synth.workload(name, n, seed=21))
    a = _run(ctx, data, k, chunks, scans, threads, il, store, tmp_path / "on")
    b = _run(ctx, data, k, chunks, scans, threads, il, "fastq", tmp_path / "off")
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        assert np.array_equal(x, y)
    on = sorted(p.name for p in (tmp_path / "on").iterdir())
    off = sorted(p.name for p in (tmp_path / "off").iterdir())
    assert on == off and any(x.endswith("_enum.bin") for x in on)
    for f in on:
        assert (tmp_path / "on" / f).read_bytes() == (tmp_path / "off" / f).read_bytes(), f


def test_packed_store_falls_back_on_other_bytes(ctx, tmp_path):
    data = bytearray(synth.fastq_bytes(synth.workload("plain_small", 4000, seed=5)))
    at = data.index(b"\n") + 5  # a base of the first read becomes lower case
    data[at] = data[at] | 0x20
    data = bytes(data)
    fno, ofs = native.fastq_index(4, [data])
    starts = native.chunk_starts_of(fno, ofs, [len(data)])
    with native.Job(ctx) as job:
        job.set_read_store("packed")
        job.load(data)
        job.count(27, starts)
        assert job.read_store == "fastq"
    a = _run(ctx, data, 27, 4, 1, 2, False, "packed", tmp_path / "on")
    b = _run(ctx, data, 27, 4, 1, 2, False, "fastq", tmp_path / "off")
    assert a[0] == b[0] and all(np.array_equal(x, y) for x, y in zip(a[1:], b[1:]))


def test_packed_store_in_upload_segments(ctx):
    import torch
    data = synth.fastq_bytes(synth.workload("plain_large", 60000, seed=8))
    host = torch.empty(len(data), dtype=torch.uint8, pin_memory=True)
    host.numpy()[:] = np.frombuffer(data, dtype=np.uint8)
    fno, ofs = native.fastq_index(32, [data])
    starts = native.chunk_starts_of(fno, ofs, [len(data)])
    res = {}
    for store in ("packed", "fastq"):
        with native.Job(ctx) as job:
            job.set_read_store(store)
            cnt = job.load_count(host.data_ptr(), len(data), 31, starts)
            if store == "packed":
                assert job.read_store == "packed" and job.kmer_cache_pieces > 1
            b = job.partition(31, 2, 8, starts, cnt.chunk_first_read, cnt.hist)
            out, sizes = job.output()
            res[store] = (b.copy(), job.labels(), bytes(out))
    a, b = res["packed"], res["fastq"]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]
