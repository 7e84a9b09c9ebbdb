"""GPU parity: the drop-in programs backed by libmetapart_gpu.so against the CPU oracle, byte for byte.

Every stage output the reference produces is compared: .idx / .KmerIdx / .kmerHist files, the enumerated,
sorted and filtered tuple streams of every scan, the BAD flags, the compressed parent array after every scan,
the parent array and component sizes before and after the mate union, and all 16 x T partition files.
"""
import pytest

import pipeline_util as pu
from metapart_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = [
    ("plain_small", 20000, pu.Params(k=27, chunks=4, scans=1, threads=2)),
    ("plain_small", 20000, pu.Params(k=27, chunks=8, scans=2, threads=4)),
    ("plain_small", 12000, pu.Params(k=27, chunks=6, scans=3, threads=3)),
    ("plain_small", 20000, pu.Params(k=31, chunks=4, scans=1, threads=1)),
    ("plain_large", 30000, pu.Params(k=31, chunks=4, scans=2, threads=2)),
    ("plain_large", 30000, pu.Params(k=29, chunks=8, scans=1, threads=8)),
    ("min3", 8000, pu.Params(k=31, chunks=4, scans=1, threads=2, min3=True)),
    ("plain_small", 20000, pu.Params(k=21, chunks=4, scans=1, threads=2, min3=True)),
    ("hotspot", 60000, pu.Params(k=31, chunks=4, scans=1, threads=2)),
    ("hotspot", 40000, pu.Params(k=25, chunks=6, scans=2, threads=3)),
    ("plain_small", 20000, pu.Params(k=11, chunks=4, scans=2, threads=2)),
    ("plain_small", 20000, pu.Params(k=13, chunks=4, scans=1, threads=4)),
    ("interleaved_small", 20000, pu.Params(k=27, chunks=4, scans=1, threads=2, interleaved=True)),
    ("interleaved_small", 20000, pu.Params(k=25, chunks=8, scans=2, threads=2, interleaved=True)),
    # many thread ranges over few reads: empty ranges, ranges of one bucket, 256 threads (the most)
    ("plain_small", 3000, pu.Params(k=27, chunks=64, scans=1, threads=64, buffer=1 << 24)),
    ("plain_large", 6000, pu.Params(k=31, chunks=128, scans=2, threads=128, buffer=1 << 24)),
    ("plain_small", 4000, pu.Params(k=23, chunks=256, scans=3, threads=256, buffer=1 << 24)),
    # the smallest inputs: one pair of reads (one or two scans), two pairs over two threads
    ("plain_small", 2, pu.Params(k=27, chunks=1, scans=1, threads=1)),
    ("plain_small", 2, pu.Params(k=21, chunks=1, scans=2, threads=1)),
    ("plain_small", 4, pu.Params(k=31, chunks=2, scans=1, threads=2)),
]

# The oracle also writes the compSizes array after every scan; the reference accumulates it without
# resetting between scans and nothing reads it before the final reset, so only the sizes at the mate
# union and after it are compared.  The parent array inside the mate union (pe_parent) holds the
# uncompressed chains of one particular union order; its compressed form is stats<S+1>_parent.
SKIP = {"dump/pe_parent.bin"}


def _keys(res, p):
    ks = [k for k in res if not k.startswith("dump/")]
    for s in range(p.scans):
        ks += [f"dump/scan{s}_enum.bin", f"dump/scan{s}_sorted.bin", f"dump/scan{s}_filtered.bin",
               f"dump/scan{s}_bad.bin", f"dump/stats{s}_parent.bin"]
    ks += [f"dump/stats{p.scans}_parent.bin", f"dump/stats{p.scans}_sizes.bin",
           f"dump/stats{p.scans + 1}_parent.bin", f"dump/stats{p.scans + 1}_sizes.bin"]
    return ks


def _compare(tmp_path, name, n, p, env_extra=None, skip=()):
    fq = tmp_path / "in.fastq"
    synth.write_fastq(synth.workload(name, n, seed=11), fq)
    do = pu.run("oracle", tmp_path, [fq], p)
    dg = pu.run("gpu", tmp_path, [fq], p, env_extra=env_extra)
    a, b = pu.outputs(do, p, "in.fastq"), pu.outputs(dg, p, "in.fastq")
    keys = [x for x in _keys(a, p) if x not in skip]
    missing = [k for k in keys if k not in b]
    assert not missing, f"GPU run did not produce {missing}"
    diff = pu.diff_keys(a, b, keys)
    assert not diff, f"GPU output differs from the oracle in {diff}"


@pytest.mark.parametrize("name,n,p", CASES, ids=[f"{c[0]}-k{c[2].k}-s{c[2].scans}-t{c[2].threads}" for c in CASES])
def test_gpu_matches_oracle(tmp_path, built_gpu, name, n, p):
    _compare(tmp_path, name, n, p)


# Narrower unit-sort digits: a different pass plan for every bucket unit.
NARROW = [
    ("plain_large", 30000, pu.Params(k=31, chunks=4, scans=2, threads=2)),
    ("hotspot", 40000, pu.Params(k=27, chunks=4, scans=1, threads=2)),
]


@pytest.mark.parametrize("bits", [5, 8])
@pytest.mark.parametrize("name,n,p", NARROW, ids=[f"{c[0]}-k{c[2].k}" for c in NARROW])
def test_gpu_unit_sort_digit_width(tmp_path, built_gpu, name, n, p, bits):
    _compare(tmp_path, name, n, p, env_extra={"MP_UNIT_SORT_MAX_BITS": str(bits)})


# The bucket's bytes as digits (three passes for a scan over half the bucket range) instead of the passes of
# near-equal widths of at most 8 bits that the sort takes by default.
@pytest.mark.parametrize("name,n,p", NARROW + [CASES[2], CASES[10]],
                         ids=[f"{c[0]}-k{c[2].k}-s{c[2].scans}" for c in NARROW + [CASES[2], CASES[10]]])
def test_gpu_byte_bucket_digits(tmp_path, built_gpu, name, n, p):
    _compare(tmp_path, name, n, p, env_extra={"MP_SORT_BUCKET_DIGITS": "bytes"})


# Scans split into bucket-range pieces (at most this many tuples in HBM at once): every stage output but
# the enumeration order, which the pieces change, equals the oracle's whole-scan run.
PIECES = [
    ("plain_large", 30000, pu.Params(k=31, chunks=4, scans=2, threads=2), 300000),
    ("plain_small", 20000, pu.Params(k=27, chunks=4, scans=1, threads=2), 100000),
    ("plain_small", 12000, pu.Params(k=27, chunks=6, scans=3, threads=3), 50000),
    ("hotspot", 40000, pu.Params(k=25, chunks=6, scans=2, threads=3), 200000),
    ("interleaved_small", 20000, pu.Params(k=25, chunks=8, scans=2, threads=2, interleaved=True), 150000),
    ("plain_small", 20000, pu.Params(k=13, chunks=4, scans=1, threads=4), 120000),
]


@pytest.mark.parametrize("name,n,p,cap", PIECES, ids=[f"{c[0]}-k{c[2].k}-s{c[2].scans}-cap{c[3]}" for c in PIECES])
def test_gpu_scan_in_pieces(tmp_path, built_gpu, name, n, p, cap):
    _compare(tmp_path, name, n, p, env_extra={"MP_SCAN_PIECE_TUPLES": str(cap)},
             skip={f"dump/scan{s}_enum.bin" for s in range(p.scans)})


# Two input files of one sample (numSE = 2, or numInterleaved = 2): reads numbered across the files, the
# index and histogram named after the first file, every partition file holding records of both.
TWO_FILES = [
    ("plain_small", "plain_large", 6000, 4000, pu.Params(k=27, chunks=8, scans=2, threads=4)),
    ("plain_small", "plain_large", 5000, 3000, pu.Params(k=31, chunks=6, scans=1, threads=3)),
    ("interleaved_small", "interleaved_small", 4000, 6000, pu.Params(k=25, chunks=4, scans=1, threads=2,
                                                                      interleaved=True)),
]


@pytest.mark.parametrize("w1,w2,n1,n2,p", TWO_FILES, ids=[f"{c[0]}+{c[1]}-k{c[4].k}-s{c[4].scans}" for c in TWO_FILES])
def test_gpu_matches_oracle_two_files(tmp_path, built_gpu, w1, w2, n1, n2, p):
    f1, f2 = tmp_path / "a.fastq", tmp_path / "b.fastq"
    synth.write_fastq(synth.workload(w1, n1, seed=3), f1)
    synth.write_fastq(synth.workload(w2, n2, seed=4), f2)
    do = pu.run("oracle", tmp_path, [f1, f2], p)
    dg = pu.run("gpu", tmp_path, [f1, f2], p)
    a, b = pu.outputs(do, p, "a.fastq"), pu.outputs(dg, p, "a.fastq")
    keys = [x for x in _keys(a, p) if x not in SKIP]
    assert not [k for k in keys if k not in b]
    assert not pu.diff_keys(a, b, keys)
