"""The allocation-free sort entry point against the allocating one.

mp_sort_tuples_noalloc exists for callers that cannot allocate device memory while they run (a host that
hands the library only buffers from its own allocator, or a loop that must not call cudaMalloc/cudaFree
between steps); its scratch is a fixed array inside the library.  Here it is called through the C ABI twice
in a row -- different sizes, with and without the high k-mer byte -- and each result must equal
mp_sort_tuples' bit for bit; then a size above its fixed limit must be refused.  The test buffers come from
torch; the entry point itself allocates nothing.  This file is collected last so that a run stopping at the
first failure has run every other test first.
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


def _inputs(n, k, seed):
    import torch
    rng = np.random.default_rng(seed)
    kmer = rng.integers(0, 1 << (2 * k), size=n, dtype=np.uint64)
    kmer[rng.integers(0, n, size=n // 4)] = kmer[0]          # ties across the tuple set
    adj = rng.integers(0, 256, size=n, dtype=np.uint64)
    ids = rng.integers(0, 1 << 31, size=n, dtype=np.uint32)
    lo = torch.from_numpy(((kmer << np.uint64(8)) | adj).view(np.int64)).cuda()
    hi = torch.from_numpy((kmer >> np.uint64(56)).astype(np.uint8)).cuda() if 2 * k + 8 > 64 else None
    return lo, hi, torch.from_numpy(ids.view(np.int32)).cuda()


def _ptr(t):
    return t.data_ptr() if t is not None else None


def test_noalloc_sort_equals_sort_on_two_calls(built_gpu):
    import torch
    f = _noalloc()
    with native.Context(0) as ctx:
        for n, k, seed in [(LIMIT, 31, 101), (300_001, 27, 102)]:
            lo, hi, ids = _inputs(n, k, seed)
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


def test_noalloc_sort_refuses_sizes_above_its_scratch(built_gpu):
    import torch
    f = _noalloc()
    t = torch.zeros(8, dtype=torch.int64, device="cuda")
    u = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = f(t.data_ptr(), None, u.data_ptr(), t.data_ptr(), None, u.data_ptr(), LIMIT + 1, None)
    assert rc == -1
    assert b"1048576" in native.lib().mp_last_error()
