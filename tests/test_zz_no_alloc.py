"""The allocation-free sort entry point against the allocating one and against a host stable sort.

mp_sort_tuples_noalloc exists for callers that cannot allocate device memory while they run (a host that
hands the library only buffers from its own allocator, or a loop that must not call cudaMalloc/cudaFree
between steps); its scratch is a fixed array inside the library.  Here it is called through the C ABI twice
in a row -- different sizes, with and without the high k-mer byte -- and each result must equal
mp_sort_tuples' and numpy's stable sort bit for bit.  Small and degenerate inputs (no tuple, one tuple, all
keys equal, which takes its no-pass branch), in-place calls with an odd and an even number of digit
passes, and the refusals (a size above its fixed limit, an output overlapping another input) follow.  The
test buffers come from torch; the entry point itself allocates nothing.  This file is collected last so
that a run stopping at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

from metapart_gb300 import native

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20


def _noalloc():
    f = native.lib().mp_sort_tuples_noalloc
    f.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _host(n, k, seed, equal=False):
    rng = np.random.default_rng(seed)
    kmer = rng.integers(0, 1 << (2 * k), size=n, dtype=np.uint64)
    if n:
        kmer[rng.integers(0, n, size=n // 4)] = kmer[0]          # ties across the tuple set
    adj = rng.integers(0, 256, size=n, dtype=np.uint64)
    if equal and n:
        kmer[:] = kmer[0]
        adj[:] = adj[0]
    ids = rng.integers(0, 1 << 31, size=n, dtype=np.uint32)
    lo = (kmer << np.uint64(8)) | adj
    hi = (kmer >> np.uint64(56)).astype(np.uint8) if 2 * k + 8 > 64 else None
    return lo, hi, ids


def _dev(lo, hi, ids):
    import torch
    d_lo = torch.from_numpy(lo.view(np.int64).copy()).cuda()
    d_hi = torch.from_numpy(hi.copy()).cuda() if hi is not None else None
    return d_lo, d_hi, torch.from_numpy(ids.view(np.int32).copy()).cuda()


def _stable_host_sort(lo, hi, ids):
    order = np.lexsort((lo, hi)) if hi is not None else np.argsort(lo, kind="stable")
    return lo[order], (hi[order] if hi is not None else None), ids[order]


def _ptr(t):
    return t.data_ptr() if t is not None else None


def _np(t, dtype):
    return t.cpu().numpy().view(dtype)


def _check_host(got_lo, got_hi, got_id, want):
    w_lo, w_hi, w_id = want
    assert np.array_equal(_np(got_lo, np.uint64), w_lo)
    assert np.array_equal(_np(got_id, np.uint32), w_id)
    if w_hi is not None:
        assert np.array_equal(_np(got_hi, np.uint8), w_hi)


def test_noalloc_sort_equals_sort_on_two_calls(built_gpu):
    import torch
    f = _noalloc()
    with native.Context(0) as ctx:
        for n, k, seed in [(LIMIT, 31, 101), (300_001, 27, 102)]:
            h = _host(n, k, seed)
            lo, hi, ids = _dev(*h)
            a_lo, a_id = torch.empty_like(lo), torch.empty_like(ids)
            a_hi = torch.empty_like(hi) if hi is not None else None
            native.sort_tuples(ctx, lo.data_ptr(), _ptr(hi), ids.data_ptr(), a_lo.data_ptr(), _ptr(a_hi),
                               a_id.data_ptr(), n)
            b_lo, b_id = torch.full_like(lo, -1), torch.full_like(ids, -1)
            b_hi = torch.full_like(hi, 0xFF) if hi is not None else None
            rc = f(lo.data_ptr(), _ptr(hi), ids.data_ptr(), b_lo.data_ptr(), _ptr(b_hi), b_id.data_ptr(), n, None)
            assert rc == 0, native.lib().mp_last_error()
            assert torch.equal(a_lo, b_lo) and torch.equal(a_id, b_id)
            if hi is not None:
                assert torch.equal(a_hi, b_hi)
            _check_host(b_lo, b_hi, b_id, _stable_host_sort(*h))


@pytest.mark.parametrize("n,k,equal", [(0, 31, False), (1, 31, False), (1, 27, False), (5000, 31, True),
                                       (5000, 27, True), (4097, 31, False)],
                         ids=["empty", "one-hi", "one", "equal-hi", "equal", "two-tiles"])
def test_noalloc_sort_small_and_degenerate(built_gpu, n, k, equal):
    import torch
    f = _noalloc()
    h = _host(n, k, 7 + n, equal)
    lo, hi, ids = _dev(*h)
    if n == 0:  # zero-length tensors may have no storage: give the call real (unused) device addresses
        lo, ids = torch.zeros(1, dtype=torch.int64, device="cuda"), torch.zeros(1, dtype=torch.int32, device="cuda")
        hi = torch.zeros(1, dtype=torch.uint8, device="cuda") if 2 * k + 8 > 64 else None
    b_lo, b_id = torch.full_like(lo, -1), torch.full_like(ids, -1)
    b_hi = torch.full_like(hi, 0xFF) if hi is not None else None
    for _ in range(2):
        rc = f(lo.data_ptr(), _ptr(hi), ids.data_ptr(), b_lo.data_ptr(), _ptr(b_hi), b_id.data_ptr(), n, None)
        assert rc == 0, native.lib().mp_last_error()
        if n:
            _check_host(b_lo, b_hi, b_id, _stable_host_sort(*h))
        else:
            assert int(b_lo[0]) == -1 and int(b_id[0]) == -1  # nothing written


@pytest.mark.parametrize("k", [31, 27], ids=["odd-passes", "even-passes"])
def test_noalloc_sort_in_place(built_gpu, k):
    f = _noalloc()
    h = _host(200_003, k, 55)
    lo, hi, ids = _dev(*h)
    rc = f(lo.data_ptr(), _ptr(hi), ids.data_ptr(), lo.data_ptr(), _ptr(hi), ids.data_ptr(), len(h[0]), None)
    assert rc == 0, native.lib().mp_last_error()
    _check_host(lo, hi, ids, _stable_host_sort(*h))


def test_noalloc_sort_refuses_sizes_above_its_scratch(built_gpu):
    import torch
    f = _noalloc()
    t = torch.zeros(8, dtype=torch.int64, device="cuda")
    u = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = f(t.data_ptr(), None, u.data_ptr(), t.data_ptr(), None, u.data_ptr(), LIMIT + 1, None)
    assert rc == -1
    assert b"1048576" in native.lib().mp_last_error()


def test_noalloc_sort_refuses_overlapping_arrays(built_gpu):
    import torch
    f = _noalloc()
    n = 1000
    lo = torch.zeros(2 * n, dtype=torch.int64, device="cuda")
    ids = torch.zeros(n, dtype=torch.int32, device="cuda")
    out_id = torch.zeros(n, dtype=torch.int32, device="cuda")
    # the keys' output starts half way into their input
    rc = f(lo.data_ptr(), None, ids.data_ptr(), lo.data_ptr() + 8 * (n // 2), None, out_id.data_ptr(), n, None)
    assert rc == -1
    assert b"overlaps" in native.lib().mp_last_error()
    # the ids' output is the keys' input
    rc = f(lo.data_ptr(), None, ids.data_ptr(), lo.data_ptr() + 8 * n, None, lo.data_ptr(), n, None)
    assert rc == -1
