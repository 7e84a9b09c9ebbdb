"""The self-checks (mp_job_set_checks, MP_CHECK=1) and the unsortedness count they use.

With the checks on, jobs of several shapes (whole scans, scans in pieces, the 3-minimizer variant) pass
them and give the results of the same job without them.  mp_count_unsorted is compared with a host count
on sorted arrays (0), on arrays with planted swaps, and on random ones, with and without the high k-mer
byte; the planted mistakes are in the input data, never in the GPU's execution.
"""
import numpy as np
import pytest

from metapart_gb300 import native, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


def _job(ctx, data, k, chunks, scans, threads, checks, cap=0, min3=False):
    fno, ofs = native.fastq_index(chunks, [data])
    starts = native.chunk_starts_of(fno, ofs, [len(data)])
    with native.Job(ctx) as job:
        job.set_checks(checks)
        job.set_scan_piece_tuples(cap)
        job.load(data)
        cnt = job.count(k, starts, min3)
        b = job.partition(k, scans, threads, starts, cnt.chunk_first_read, cnt.hist, min3)
        out, sizes = job.output()
        return b.copy(), job.labels(), bytes(out), job.scan_pieces


@pytest.mark.parametrize("name,n,k,scans,cap,min3", [("plain_large", 40000, 31, 2, 0, False),
                                                    ("plain_small", 30000, 27, 1, 0, False),
                                                    ("plain_large", 40000, 31, 2, 300000, False),
                                                    ("min3", 20000, 31, 1, 0, True)],
                         ids=["k31-s2", "k27-s1", "pieces", "min3"])
def test_checks_pass_and_change_nothing(ctx, name, n, k, scans, cap, min3):
    data = synth.fastq_bytes(synth.workload(name, n, seed=61))
    a = _job(ctx, data, k, 16, scans, 4, True, cap, min3)
    b = _job(ctx, data, k, 16, scans, 4, False, cap, min3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]
    if cap:
        assert a[3] > scans


def _host_unsorted(lo, hi):
    key_hi = hi.astype(np.uint64) if hi is not None else np.zeros_like(lo)
    a_hi, b_hi, a_lo, b_lo = key_hi[:-1], key_hi[1:], lo[:-1], lo[1:]
    return int(np.count_nonzero((a_hi > b_hi) | ((a_hi == b_hi) & (a_lo > b_lo))))


@pytest.mark.parametrize("with_hi", [False, True], ids=["lo", "lo+hi"])
def test_count_unsorted_matches_the_host(ctx, with_hi):
    import torch
    rng = np.random.default_rng(5)
    n = 1_000_003
    lo = np.sort(rng.integers(0, 1 << 62, size=n, dtype=np.uint64))
    hi = np.zeros(n, dtype=np.uint8) if with_hi else None
    if with_hi:  # a sorted (hi, lo) order: hi ascending in blocks, lo sorted within each
        hi = np.sort(rng.integers(0, 64, size=n, dtype=np.uint8))
        for v in np.unique(hi):
            m = hi == v
            lo[m] = np.sort(lo[m])
    cases = [("sorted", lo.copy(), None if hi is None else hi.copy())]
    swapped = lo.copy()
    idx = rng.choice(n - 1, size=37, replace=False)
    for i in idx:
        swapped[i], swapped[i + 1] = swapped[i + 1], swapped[i]
    cases.append(("swaps", swapped, None if hi is None else hi.copy()))
    cases.append(("random", rng.integers(0, 1 << 62, size=n, dtype=np.uint64),
                  None if hi is None else rng.integers(0, 64, size=n, dtype=np.uint8)))
    for name, l, h in cases:
        d_lo = torch.from_numpy(l.view(np.int64)).cuda()
        d_hi = torch.from_numpy(h).cuda() if h is not None else None
        got = native.count_unsorted(ctx, d_lo.data_ptr(), d_hi.data_ptr() if d_hi is not None else None, n)
        assert got == _host_unsorted(l, h), name
    assert native.count_unsorted(ctx, 0, None, 0) == 0
