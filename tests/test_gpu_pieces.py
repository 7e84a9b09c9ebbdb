"""Scans split into bucket-range pieces through the job API: a job told to hold fewer tuples at once than a
scan has runs the scan in pieces of consecutive m-mer buckets and gives the labels, bounds and partition
files of the whole scans (with the count pass's k-mer cache, and without it).  The 3-minimizer variant,
whose minimizer choice depends on the bucket range, is never split."""
import numpy as np
import pytest

from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu

# (workload, reads, k, chunks, scans, threads, interleaved, most tuples at once)
CASES = [
    ("plain_large", 40000, 31, 16, 2, 4, False, 400000),
    ("interleaved_small", 30000, 27, 16, 2, 2, True, 200000),
    ("hotspot", 30000, 25, 12, 1, 2, False, 150000),
    ("plain_small", 20000, 21, 8, 3, 2, False, 60000),
]


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


def _run(ctx, data, k, chunks, scans, threads, il, cap, kc=True, min3=False):
    fno, ofs = native.fastq_index(chunks, [data], il)
    starts = native.chunk_starts_of(fno, ofs, [len(data)])
    job = native.Job(ctx)
    try:
        job.set_kmer_cache(kc)
        job.set_scan_piece_tuples(cap)
        job.load(data, interleaved=il)
        cnt = job.count(k, starts, min3)
        bounds = job.partition(k, scans, threads, starts, cnt.chunk_first_read, cnt.hist, min3)
        out, sizes = job.output()
        return dict(bounds=bounds.copy(), labels=job.labels(), out=bytes(out), sizes=sizes.copy(),
                    pieces=job.scan_pieces)
    finally:
        job.close()


def _same(a, b):
    for key in ("bounds", "labels", "sizes"):
        assert np.array_equal(a[key], b[key]), key
    assert a["out"] == b["out"]


@pytest.mark.parametrize("name,n,k,chunks,scans,threads,il,cap", CASES,
                         ids=[f"{c[0]}-k{c[2]}-s{c[4]}" for c in CASES])
def test_pieces_equal_whole_scans(ctx, name, n, k, chunks, scans, threads, il, cap):
    data = synth.fastq_bytes(synth.workload(name, n, seed=51))
    whole = _run(ctx, data, k, chunks, scans, threads, il, 0)
    split = _run(ctx, data, k, chunks, scans, threads, il, cap)
    assert whole["pieces"] == scans and split["pieces"] > scans
    _same(split, whole)


def test_pieces_without_kmer_cache(ctx):
    data = synth.fastq_bytes(synth.workload("plain_large", 30000, seed=52))
    whole = _run(ctx, data, 31, 8, 2, 2, False, 0, kc=False)
    split = _run(ctx, data, 31, 8, 2, 2, False, 250000, kc=False)
    assert split["pieces"] > 2
    _same(split, whole)


def test_buckets_above_the_cap(ctx):
    """A cap below the hot buckets' counts: each of those is a piece of its own (with the empty buckets
    before it)."""
    data = synth.fastq_bytes(synth.workload("hotspot", 30000, seed=53))
    whole = _run(ctx, data, 27, 4, 1, 2, False, 0)
    split = _run(ctx, data, 27, 4, 1, 2, False, 20000)
    assert split["pieces"] > 100
    _same(split, whole)


def test_min3_is_not_split(ctx):
    data = synth.fastq_bytes(synth.workload("plain_small", 20000, seed=54))
    whole = _run(ctx, data, 31, 8, 1, 2, False, 0, min3=True)
    split = _run(ctx, data, 31, 8, 1, 2, False, 1000, min3=True)
    assert split["pieces"] == 1
    _same(split, whole)
