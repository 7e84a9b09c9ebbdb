"""Model check of the parallel mate union (the round structure of k_pe_reserve / k_pe_commit /
k_pe_bigsmall) against the reference's in-order loop (metapart.c:2801-2867) on random forests, including
components above the 1000-read limit.  The model follows the kernels step by step: roots and sizes are read
at the start of a round, a pair commits when it holds the reservation of each of its small roots, large
roots are shared and end under the maximum root of their group."""
import random

import pytest

LIMIT = 1000


def sequential(parent, size):
    parent, size = parent[:], size[:]

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x
    for i in range(0, len(parent), 2):
        a, b = find(i), find(i + 1)
        if (size[a] <= LIMIT or size[b] <= LIMIT) and a != b:
            hi, lo = max(a, b), min(a, b)
            parent[lo] = hi
            size[hi] += size[lo]
            size[lo] = 0
    return [find(x) for x in range(len(parent))]


def rounds(parent, size):
    parent, size = parent[:], size[:]

    def find(x):
        while parent[x] != x:
            x = parent[x]
        return x
    act = list(range(len(parent) // 2))
    n_rounds = 0
    while act:
        n_rounds += 1
        resv, surv, snap = {}, [], {}
        for j in act:                                  # k_pe_reserve
            ra, rb = find(2 * j), find(2 * j + 1)
            if ra == rb:
                continue
            za, zb = size[ra], size[rb]
            if za > LIMIT and zb > LIMIT:
                continue
            snap[j] = (ra, rb, za, zb)
            surv.append(j)
            for r, z in ((ra, za), (rb, zb)):
                if z <= LIMIT:
                    resv[r] = min(resv.get(r, 1 << 62), j)
        if not surv:
            break
        nxt, big, gmax, gadd = [], [], {}, {}
        for j in surv:                                 # k_pe_commit
            ra, rb, za, zb = snap[j]
            sa, sb = za <= LIMIT, zb <= LIMIT
            if not ((not sa or resv[ra] == j) and (not sb or resv[rb] == j)):
                nxt.append(j)
                continue
            if sa and sb:
                hi, lo = max(ra, rb), min(ra, rb)
                parent[lo] = hi
                size[hi] = za + zb
                size[lo] = 0
            else:
                g, x, zx = (rb, ra, za) if sa else (ra, rb, zb)
                gmax[g] = max(gmax.get(g, -1), x)
                gadd[g] = gadd.get(g, 0) + zx
                big.append((g, x))
        for g, x in big:                               # k_pe_bigsmall
            mx = gmax[g]
            R = max(mx, g)
            if x != mx:
                parent[x] = R
                size[x] = 0
                continue
            tot = size[g] + gadd[g]
            if R != g:
                parent[g] = R
                size[g] = 0
            else:
                parent[x] = R
                size[x] = 0
            size[R] = tot
        act = nxt
    return [find(x) for x in range(len(parent))], n_rounds


def random_forest(n, seed, big_frac):
    rnd = random.Random(seed)
    parent = list(range(n))
    ids = list(range(n))
    rnd.shuffle(ids)
    p = 0
    while p < n:
        s = rnd.choice([1, 1, 1, 2, 3, 5, 20, 200, 999, 1000, 1001]) if rnd.random() > big_frac else rnd.randrange(
            1000, 3000)
        grp = ids[p:p + s]
        r = max(grp)
        for x in grp:
            parent[x] = r
        p += s
    size = [0] * n
    for x in range(n):
        size[parent[x]] += 1
    return parent, size


@pytest.mark.parametrize("n,seed,big", [(2000, 1, 0.0), (6000, 2, 0.1), (20000, 3, 0.3), (40000, 4, 0.05),
                                         (12000, 5, 0.5)])
def test_rounds_equal_sequential(n, seed, big):
    parent, size = random_forest(n, seed, big)
    want = sequential(parent, size)
    got, nr = rounds(parent, size)
    assert got == want
    assert nr < n
