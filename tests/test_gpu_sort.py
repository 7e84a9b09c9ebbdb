"""mp_sort_tuples (the onesweep radix sort on device pointers) against a stable host sort by (k-mer, adjacency)
on seeded tuples: random keys, heavy ties, constant high digits (skipped passes), 2k + 8 > 64 keys."""
import numpy as np
import pytest

from metapart_gb300 import native

pytestmark = pytest.mark.gpu


def host_sort(kmer, adj, ids):
    order = np.lexsort((adj, kmer))   # stable: ties keep input order
    return kmer[order], adj[order], ids[order]


@pytest.fixture(scope="module")
def ctx(built_gpu):
    c = native.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("n,k,ties,seed", [(1, 27, False, 1), (4095, 27, False, 2), (4097, 31, True, 3),
                                           (300_000, 31, False, 4), (250_000, 27, True, 5), (1_000_003, 29, False, 6)])
def test_sort_matches_stable_host_sort(ctx, n, k, ties, seed):
    import torch
    rng = np.random.default_rng(seed)
    top = 1 << (2 * k)
    kmer = rng.integers(0, 64 if ties else top, size=n, dtype=np.uint64)
    if not ties:
        kmer &= np.uint64(top - 1)
    adj = rng.integers(0, 256, size=n, dtype=np.uint64) if not ties else rng.integers(0, 3, size=n, dtype=np.uint64)
    ids = rng.integers(0, 1 << 31, size=n, dtype=np.uint32)
    has_hi = 2 * k + 8 > 64
    lo = (kmer << np.uint64(8)) | adj
    hi = (kmer >> np.uint64(56)).astype(np.uint8)
    d_lo, d_id = torch.from_numpy(lo.view(np.int64)).cuda(), torch.from_numpy(ids.view(np.int32)).cuda()
    d_hi = torch.from_numpy(hi).cuda() if has_hi else None
    o_lo, o_id = torch.empty_like(d_lo), torch.empty_like(d_id)
    o_hi = torch.empty_like(d_hi) if has_hi else None
    native.sort_tuples(ctx, d_lo.data_ptr(), d_hi.data_ptr() if has_hi else None, d_id.data_ptr(), o_lo.data_ptr(),
                       o_hi.data_ptr() if has_hi else None, o_id.data_ptr(), n)
    g_lo = o_lo.cpu().numpy().view(np.uint64)
    g_kmer = (g_lo >> np.uint64(8)) | ((o_hi.cpu().numpy().astype(np.uint64) << np.uint64(56)) if has_hi else 0)
    wk, wa, wi = host_sort(kmer, adj, ids)
    assert np.array_equal(g_kmer, wk)
    assert np.array_equal(g_lo & np.uint64(0xFF), wa)
    assert np.array_equal(o_id.cpu().numpy().view(np.uint32), wi)
