// K4 (branching k-mer filter), K5 (run edges + union-find), K6 (mate union) and the
// partition planner, on the sorted tuples of one scan and the per-read parent array.
//
// parent[] is the reference's parent array as u32 with BAD = 0xFFFFFFFF standing for
// 0xBADBADBAD (metapart.c:2330-2340).  Components hook the smaller root under the larger
// one, so every component's root is its largest read id (metapart.c:2683-2716,
// unionfind.h:58-66) regardless of the order unions run in.
#include <algorithm>
#include <vector>

#include "k_graph.cuh"

namespace mp {

constexpr int SEG = 1024;          // tuples owned by one warp in the run kernels
constexpr uint32_t UF_CAP = 1u << 20;
constexpr unsigned FULLW = 0xFFFFFFFFu;

__device__ __forceinline__ uint64_t kmer_of(const uint64_t *lo, const uint8_t *hi, uint64_t i)
{
    return (lo[i] >> 8) | (hi ? ((uint64_t)hi[i] << 56) : 0ull);
}

__device__ __forceinline__ bool zbit(const uint32_t *z, uint64_t i) { return (z[i >> 5] >> (i & 31)) & 1u; }

// e is a thread-range end (the reference never judges the last run of a range, metapart.c:2289-2467)
__device__ __forceinline__ bool at_range_end(const uint64_t *ends, int T, uint64_t e)
{
    int lo = 0, hi = T - 1;
    while (lo <= hi) {
        int m = (lo + hi) >> 1;
        if (ends[m] == e) return true;
        if (ends[m] < e) lo = m + 1; else hi = m - 1;
    }
    return false;
}

// lanes [s, e) of a window (s <= 31, e <= 32)
__device__ __forceinline__ uint32_t lane_range(int s, int e)
{
    const uint32_t hi = e >= 32 ? FULLW : ((1u << e) - 1);
    return hi & ~((1u << s) - 1);
}

// --------------------------------------------------------------- K4 filter

// Decision of markMischiefKmers for one run (metapart.c:2296-2451), packed:
// bit 0 branching (numIn > 1 or numOut > 1), 1 numIn > 1, 2 numOut > 1, 3-5 max in index,
// 6-8 max out index, 9 zero the k-mer (both sides branch), 10 second-max ratio above 0.2.
constexpr uint32_t J_ANY = 1, J_NIN = 2, J_NOUT = 4, J_ZERO = 1u << 9, J_RATIO = 1u << 10;

// The reference's test (float)s / deg > 0.2, the float quotient compared as a double
// (metapart.c:2346-2349).  The smallest float above 0.2 is 0.2f = 13421773 * 2^-26, and a
// quotient rounds to at least that iff it exceeds the midpoint 26843545 * 2^-27 (a tie
// rounds to the even neighbour below), so for s, deg exact in float (<= 2^24) the test is
// s * 2^27 > 26843545 * deg in integers -- no FP64, which is slow on this GPU.
__device__ __forceinline__ bool ratio_above_02(uint32_t s, uint32_t deg)
{
    if (deg <= (1u << 24)) return ((uint64_t)s << 27) > 26843545ull * deg;
    return (double)__fdiv_rn((float)s, (float)deg) > 0.2;
}

__device__ __forceinline__ uint32_t judge_run(const uint32_t *before, const uint32_t *after, uint32_t deg)
{
    int nin = 0, nout = 0, mxi = 0, mxo = 0;
    uint32_t cmi = 0, cmo = 0, smi = 0, smo = 0;
    // the first code with the largest count is the max; a count equal to it is the second max
#pragma unroll
    for (int q = 0; q < 7; q++) {
        const uint32_t b = before[q], a = after[q];
        const bool gb = b > cmi, ga = a > cmo;
        nin += b != 0;
        nout += a != 0;
        smi = gb ? cmi : max(smi, b);
        smo = ga ? cmo : max(smo, a);
        mxi = gb ? q : mxi;
        mxo = ga ? q : mxo;
        cmi = max(cmi, b);
        cmo = max(cmo, a);
    }
    if (nin <= 1 && nout <= 1) return 0;
    uint32_t J = J_ANY | (nin > 1 ? J_NIN : 0) | (nout > 1 ? J_NOUT : 0) | ((uint32_t)mxi << 3) | ((uint32_t)mxo << 6);
    if (nin > 1 && nout > 1) J |= J_ZERO;
    if (ratio_above_02(smi, deg) || ratio_above_02(smo, deg)) J |= J_RATIO;
    return J;
}

// Marks of one tuple of a judged run: the zero flag goes to the z bitmask (the tuple array
// stays read-only while other warps detect run heads), BAD to the read.
__device__ __forceinline__ void mark_tuple(uint32_t J, uint64_t q, uint32_t adj, const uint32_t *id, uint32_t *parent,
                                           uint8_t *filtered, uint32_t *z)
{
    if (!(J & J_ANY)) return;
    if (J & J_ZERO) {
        atomicOr(&z[q >> 5], 1u << (q & 31));
        return;
    }
    const uint32_t bi = adj & 7, ai = (adj >> 3) & 7;
    bool bad = ((J & J_NIN) && bi != ((J >> 3) & 7)) || ((J & J_NOUT) && ai != ((J >> 6) & 7));
    if (!bad) bad = (J & J_RATIO) != 0;
    if (bad) {
        const uint32_t r = id[q];
        parent[r] = BAD;
        filtered[r] = 1;
    }
}

// One warp per SEG tuples: the runs whose first tuple lies in the warp's segment.  In each
// window of 32 tuples a lane finds whether its tuple starts a run (one shuffle) and whether its
// adjacency byte differs from the previous tuple of its run.  A run whose tuples all share one
// adjacency byte has at most one before- and one after-code, so markMischiefKmers leaves it alone;
// a window holding only such runs costs a few ballots.  Otherwise 14 ballots give every run its
// before/after adjacency-code counts by popcount.  A run still open at the end of a window is
// carried: while it is uniform its counts follow from its length and byte; when it spans windows
// its marks are applied by one more pass over it after it is judged.
// MULTI: the thread ranges of several scans one after another (a batch of samples), whose boundaries may
// cut a run of equal k-mers; within one scan ranges cut runs only between buckets.
template <bool MULTI>
__global__ void __launch_bounds__(256) k_filter_warp(const uint64_t *lo, const uint8_t *hi, const uint32_t *id,
                                                     uint64_t n, const uint64_t *range_ends, int T, uint32_t *parent,
                                                     uint8_t *filtered, uint32_t *z)
{
    __shared__ uint64_t ends_s[256];
    const bool in_smem = T <= 256;  // many ranges (a batch of samples) are read from global memory
    if (in_smem)
        for (int t = threadIdx.x; t < T; t += blockDim.x) ends_s[t] = range_ends[t];
    __syncthreads();
    const uint64_t *ends = in_smem ? ends_s : range_ends;
    const int lane = threadIdx.x & 31;
    const uint64_t c0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * SEG;
    if (c0 >= n) return;
    const uint64_t c1 = min(n, c0 + SEG);
    const uint32_t le = (lane == 31) ? FULLW : ((2u << lane) - 1);  // lanes <= lane
    bool open = false, ohom = true;  // a run carried into the next window; all its bytes equal so far
    uint64_t rs = 0;
    uint32_t cb[7], ca[7], deg = 0;  // its counts (kept while it is not uniform)
#pragma unroll
    for (int c = 0; c < 7; c++) cb[c] = ca[c] = 0;
    uint64_t prev_km = 0;
    uint32_t prev_adj = 0;
    if (c0) {
        const uint64_t l = lo[c0 - 1];
        prev_km = (l >> 8) | (hi ? ((uint64_t)hi[c0 - 1] << 56) : 0ull);
        prev_adj = (uint32_t)(l & 0xFF);
    }
    uint64_t nlv = c0 + lane < n ? lo[c0 + lane] : 0;  // next window's words, loaded one window ahead
    uint8_t nhv = (hi && c0 + lane < n) ? hi[c0 + lane] : 0;
    // range ends: the warp's windows advance in order, so a cursor over the sorted ends gives each window
    // the ends in [p, p + 32] as a bit mask (bit e - p)
    int ne = 0;
    {
        int lo_i = 0, hi_i = T;  // first end >= c0
        while (lo_i < hi_i) {
            const int m = (lo_i + hi_i) >> 1;
            if (ends[m] < c0) lo_i = m + 1; else hi_i = m;
        }
        ne = lo_i;
    }
    uint64_t nxt_end = ne < T ? ends[ne] : ~0ull;  // the next range end at or after the window
    for (uint64_t p = c0;; p += 32) {
        const bool owned = p < c1;
        if (!owned && !open) break;
        uint64_t emask = 0;
        while (nxt_end < p + 32) {
            emask |= 1ull << (nxt_end - p);
            nxt_end = ++ne < T ? ends[ne] : ~0ull;
        }
        if (nxt_end == p + 32) emask |= 1ull << 32;
        const uint64_t i = p + lane;
        const bool valid = i < n;
        const uint64_t lv = nlv;
        const uint64_t km = valid ? ((lv >> 8) | ((uint64_t)nhv << 56)) : 0;
        if (i + 32 < n) {
            nlv = lo[i + 32];
            if (hi) nhv = hi[i + 32];
        }
        const uint32_t adj = (uint32_t)(lv & 0xFF);
        uint64_t pk = __shfl_up_sync(FULLW, km, 1);
        uint32_t pa = __shfl_up_sync(FULLW, adj, 1);
        if (lane == 0) {
            pk = prev_km;
            pa = prev_adj;
        }
        // a thread range starts a run whatever the k-mer before it (each range is its own sweep)
        const bool head = valid && (i == 0 || km != pk || (MULTI && ((emask >> lane) & 1u)));
        const uint32_t H = __ballot_sync(FULLW, head), V = __ballot_sync(FULLW, valid);
        const uint32_t D = __ballot_sync(FULLW, valid && !head && adj != pa);
        const uint32_t run_adj = prev_adj;  // byte of a uniform carried run
        prev_km = __shfl_sync(FULLW, km, 31);
        prev_adj = __shfl_sync(FULLW, adj, 31);
        const int fh = H ? __ffs(H) - 1 : 32;
        const bool arr_end = p + 32 >= n;
        const int lh = H ? 31 - __clz(H) : -1;
        if (D == 0 && !(open && !ohom)) {
            // every run that ends in this window is uniform: no marks
            if (open && (fh < 32 || arr_end)) open = false;
            if (!owned) continue;
            if (lh >= 0 && !arr_end) {
                open = true;
                ohom = true;
                rs = p + lh;
            }
            continue;
        }
        if (open && ohom) {  // counts of the uniform part carried in
            const uint32_t len = (uint32_t)(p - rs), rb = run_adj & 7, ra = (run_adj >> 3) & 7;
#pragma unroll
            for (int c = 0; c < 7; c++) {  // code 7 counts nowhere; no dynamic index, so the counts stay in registers
                cb[c] = (uint32_t)c == rb ? len : 0u;
                ca[c] = (uint32_t)c == ra ? len : 0u;
            }
            deg = len;
            ohom = false;
        }
        uint32_t Bm[7], Am[7];
#pragma unroll
        for (int c = 0; c < 7; c++) {
            Bm[c] = __ballot_sync(FULLW, valid && (adj & 7) == (uint32_t)c);
            Am[c] = __ballot_sync(FULLW, valid && ((adj >> 3) & 7) == (uint32_t)c);
        }
        // the run carried into this window occupies lanes [0, fh)
        if (open) {
            const uint32_t m = lane_range(0, fh) & V;
#pragma unroll
            for (int c = 0; c < 7; c++) { cb[c] += __popc(Bm[c] & m); ca[c] += __popc(Am[c] & m); }
            deg += __popc(m);
            if (fh < 32 || arr_end) {
                const uint64_t re = fh < 32 ? p + fh : n;
                open = false;
                if (!((emask >> (re - p)) & 1u)) {
                    const uint32_t J = judge_run(cb, ca, deg);
                    if (J & J_ANY)
                        for (uint64_t q = rs + lane; q < re; q += 32) mark_tuple(J, q, (uint32_t)(lo[q] & 0xFF), id, parent, filtered, z);
                }
            }
        }
        if (!owned) continue;
        // runs that start in this window
        uint32_t J = 0;
        int s = -1;
        if (H & le) s = 31 - __clz(H & le);
        const uint32_t later = H & ~le;
        const int nh = later ? __ffs(later) - 1 : 32;
        if (head && (nh < 32 || arr_end)) {
            const uint32_t m = lane_range(lane, nh) & V;
            if (D & m) {  // a uniform run needs no judgement
                uint32_t b[7], a[7];
#pragma unroll
                for (int c = 0; c < 7; c++) { b[c] = __popc(Bm[c] & m); a[c] = __popc(Am[c] & m); }
                const uint64_t re = nh < 32 ? p + nh : n;
                if (!((emask >> (re - p)) & 1u)) J = judge_run(b, a, __popc(m));
            }
        }
        const uint32_t Js = __shfl_sync(FULLW, J, s < 0 ? 0 : s);
        if (s >= 0 && valid) mark_tuple(Js, i, adj, id, parent, filtered, z);  // J == 0 for the still-open run
        // the last run of the window stays open when the array continues past it
        if (lh >= 0 && !arr_end) {
            const uint32_t m = lane_range(lh, 32) & V;
            rs = p + lh;
            open = true;
            ohom = (D & m) == 0;
            if (!ohom) {
#pragma unroll
                for (int c = 0; c < 7; c++) { cb[c] = __popc(Bm[c] & m); ca[c] = __popc(Am[c] & m); }
                deg = __popc(m);
            }
        }
    }
}

// Applies the zero marks to the tuples (lo = adj, hi = 0): only for stage dumps.
__global__ void k_apply_zero(uint64_t *lo, uint8_t *hi, uint64_t n, const uint32_t *z)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && zbit(z, i)) {
        lo[i] &= 0xFF;
        if (hi) hi[i] = 0;
    }
}

// ---------------------------------------------------------- union-find

// The roots of x and of y, the two walks advanced together so that their parent loads are in flight at
// the same time.  A walk stops at a node that is its own parent or whose parent is BAD (a BAD read is
// its own root, unionfind.h:25-32), and halves its path as it goes (a node is pointed at its
// grandparent).  When the walks meet (the same node on both) the two are in one component: x and y come
// back equal without the rest of the walk (callers use the results as roots only when they differ).
__device__ __forceinline__ void uf_find2(uint32_t *parent, uint32_t &x, uint32_t &y)
{
    bool dx = false, dy = false;
    for (;;) {
        const uint32_t px = dx ? x : parent[x];
        const uint32_t py = dy ? y : parent[y];
        if (px == py && px != BAD) {
            x = y = px;
            return;
        }
        dx = dx || px == x || px == BAD;
        dy = dy || py == y || py == BAD;
        if (dx && dy) return;
        const uint32_t gx = dx ? x : parent[px];
        const uint32_t gy = dy ? y : parent[py];
        if (!dx) {
            if (gx == px || gx == BAD) {
                x = px;
                dx = true;
            } else {
                parent[x] = gx;  // path halving: gx is an ancestor of x
                x = gx;
            }
        }
        if (!dy) {
            if (gy == py || gy == BAD) {
                y = py;
                dy = true;
            } else {
                parent[y] = gy;
                y = gy;
            }
        }
        if (dx && dy) return;
    }
}

__device__ __forceinline__ void uf_union(uint32_t *parent, uint32_t a, uint32_t b, uint32_t *err, uint32_t cap)
{
    for (uint32_t it = 0; it < cap; it++) {
        uint32_t ra = a, rb = b;
        uf_find2(parent, ra, rb);
        if (ra == rb) return;
        const uint32_t hi = ra > rb ? ra : rb, lo = ra > rb ? rb : ra;
        if (atomicCAS(&parent[lo], lo, hi) == lo) return;
    }
    atomicOr(err, DERR_SPIN);
}

// First tuple of each thread range whose k-mer is not zero (nor zero-marked) and whose read is not BAD.
__global__ void k_range_first_valid(const uint64_t *lo, const uint8_t *hi, const uint32_t *id, const uint32_t *z,
                                    const uint64_t *range_bounds, int T, const uint32_t *parent, uint64_t *first)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    uint64_t f = ~0ull;
    for (uint64_t q = range_bounds[t]; q < range_bounds[t + 1]; q++)
        if (!zbit(z, q) && kmer_of(lo, hi, q) != 0 && parent[id[q]] != BAD) { f = q; break; }
    first[t] = f;
}

// A BAD read as a sweep's initial anchor.  A thread range's sweep starts from the scan's last k-mer and
// the scan's first read (metapart.c:2539-2545), so the run of the range's first valid tuple is united with
// that read when it carries the last k-mer, BAD or not.  findRoot returns a read whose parent is BAD as
// its own root (unionfind.h:25) and each union hooks the smaller root below the larger (:2680-2700).  So
// with a BAD first read B the run's components are hooked below B while their roots are smaller than B,
// until one is larger: B then goes below it and is a member like any other (parent no longer BAD).  If
// none is, B keeps its BAD parent and the edge replay's assertion stops the reference (:2772).  The run is
// the scan's last and the range is the last with tuples, so nothing else joins the component after it:
// the outcome is B below the component's final root when B is smaller than that root, else nothing.
// Here the run is united like any other (its first valid tuple as anchor) and B is hooked afterwards.
// At most one range of a scan has its first valid tuple in the last run (ranges end between buckets).

// The read of the range's first valid tuple when that tuple carries the scan's last k-mer (~0u stays).
__global__ void k_bad_anchor_find(const uint64_t *lo, const uint8_t *hi, const uint32_t *id, const uint64_t *first, int T,
                                  uint64_t init_kmer, uint32_t *anchor_v)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const uint64_t f = first[t];
    if (f != ~0ull && kmer_of(lo, hi, f) == init_kmer) *anchor_v = id[f];
}

__device__ __forceinline__ uint32_t root_of(const uint32_t *parent, uint32_t x)
{
    for (uint32_t it = 0; it < UF_CAP; it++) {
        const uint32_t p = parent[x];
        if (p == x || p == BAD) break;
        x = p;
    }
    return x;
}

// After the scan's unions: hooks the BAD first read below the root of the run's component when it is the
// smaller id (records it in *hooked, which the next scan marks BAD again like every flagged read).
__global__ void k_bad_anchor_hook(uint32_t *parent, uint32_t b, const uint32_t *anchor_v, uint32_t *hooked)
{
    const uint32_t v = *anchor_v;
    if (v == ~0u || parent[b] != BAD) return;
    const uint32_t r = root_of(parent, v);
    if (b < r) {
        parent[b] = r;
        *hooked = b;
    }
}

// The same for every range of a batch (each sample its own scan, its own first read and last k-mer).
__global__ void k_seg_bad_anchor(const uint64_t *lo, const uint8_t *hi, const uint32_t *id, const uint64_t *first, int R,
                                 const uint64_t *r_kmer, const uint32_t *r_min, const uint32_t *r_ok, uint32_t *parent)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= R) return;
    const uint64_t f = first[t];
    if (r_ok[t] || f == ~0ull || kmer_of(lo, hi, f) != r_kmer[t]) return;
    const uint32_t b = r_min[t];
    if (parent[b] != BAD) return;
    const uint32_t r = root_of(parent, id[f]);
    if (b < r) parent[b] = r;
}

// markMischiefKmers' closing sweep (metapart.c:2503-2516) at a later scan: a flagged read whose parent is
// not BAD gets BAD again.  Only a hooked first read (above) can be one.
__global__ void k_rebad(uint32_t *parent, uint32_t r) { parent[r] = BAD; }

struct EdgeCtx {
    const uint64_t *lo;
    const uint8_t *hi;
    const uint32_t *id;
    const uint32_t *z;             // zero marks of the filter
    uint64_t n;
    const uint64_t *first_valid;   // per thread range (~0: none)
    const uint64_t *range_bounds;  // T + 1 tuple bounds
    int T;
    uint64_t init_kmer;            // k-mer of the scan's last tuple after the filter (metapart.c:2541)
    uint32_t init_min;             // read id of the scan's first tuple (metapart.c:2543-2545)
    uint32_t init_min_ok;          // that read is not BAD
    // per thread range instead (a batch of samples, each its own scan); nullable
    const uint64_t *r_kmer;
    const uint32_t *r_min;
    const uint32_t *r_ok;
    uint32_t *parent;
    const uint8_t *filtered;       // BAD flags: during the scans a read's parent is BAD exactly when it is flagged
    uint32_t *err;
    uint32_t uf_cap;               // hook retries of one union before it gives up (DERR_SPIN)
};

// unionFindPar2 (metapart.c:2537-2727): in each run of equal k-mers the first valid tuple
// (k-mer not zero, read not BAD) is the anchor and every later valid tuple is united with it.
// For the first valid run of a thread range whose k-mer equals the scan's last k-mer, the
// anchor is the scan's first read (the sweep's initial state, :2539-2548).  One warp per
// SEG tuples, windows of 32 as in the filter; the anchor of a run still open at the end of a
// window is carried.
// MULTI: many thread ranges of several scans (a batch of samples): a range start is a run head whatever the
// k-mer before it, and every range has its own initial state (c.r_*), found by cursors over the ranges.
// Without it (one scan), ranges cut runs only between buckets and the initial state is the scan's own.
template <bool MULTI>
__global__ void __launch_bounds__(256) k_edges_warp(EdgeCtx c)
{
    const int lane = threadIdx.x & 31;
    const uint64_t c0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * SEG;
    if (c0 >= c.n) return;
    const uint64_t c1 = min(c.n, c0 + SEG);
    const uint32_t le = (lane == 31) ? FULLW : ((2u << lane) - 1);
    bool open = false, has_anchor = false;
    uint32_t anchor = 0;
    // cursors over the thread ranges: their starts (run heads) and their first valid tuples (the positions
    // where a range's sweep may take the scan's initial state); both ascend with the range index
    int nb = 0, nf = 0;
    uint64_t nxt_b = ~0ull, nxt_f = ~0ull;  // the next range start, the next range's first valid tuple
    if constexpr (MULTI) {
        int a = 1, b = c.T;  // first t in [1, T] with range_bounds[t] >= c0 (T when none)
        while (a < b) {
            const int m = (a + b) >> 1;
            if (c.range_bounds[m] < c0) a = m + 1; else b = m;
        }
        nb = a;
        a = 0, b = c.T - 1;  // the range holding c0: ranges before it have their first valid tuple below c0
        while (a < b) {
            const int m = (a + b + 1) >> 1;
            if (c.range_bounds[m] <= c0) a = m; else b = m - 1;
        }
        nf = a;
        nxt_b = nb < c.T ? c.range_bounds[nb] : ~0ull;
        nxt_f = c.first_valid[nf];
        while (nxt_f == ~0ull && ++nf < c.T) nxt_f = c.first_valid[nf];
    }
    uint64_t prev_km = c0 ? kmer_of(c.lo, c.hi, c0 - 1) : 0;
    // the next window's k-mer, read id and zero-mark word (windows start at multiples of 32), loaded one
    // window ahead
    uint64_t nkm = c0 + lane < c.n ? kmer_of(c.lo, c.hi, c0 + lane) : 0;
    uint32_t nid = c0 + lane < c.n ? c.id[c0 + lane] : 0, nzw = c.z[c0 >> 5];
    for (uint64_t p = c0;; p += 32) {
        const bool owned = p < c1;
        if (!owned && !open) break;
        const uint64_t i = p + lane;
        const bool valid = i < c.n;
        const uint64_t km = valid ? nkm : 0;
        const uint32_t rid = nid, zw = nzw;
        if (p + 32 < c.n) {
            if (i + 32 < c.n) {
                nkm = kmer_of(c.lo, c.hi, i + 32);
                nid = c.id[i + 32];
            }
            nzw = c.z[(p + 32) >> 5];
        }
        uint32_t smask = 0, fmask = 0;  // lanes at a range start, lanes at a range's first valid tuple
        int my_t = 0;                   // the range whose first valid tuple this lane holds
        while (MULTI && nxt_b < p + 32) {
            if (nxt_b >= p) smask |= 1u << (nxt_b - p);
            nxt_b = ++nb < c.T ? c.range_bounds[nb] : ~0ull;
        }
        while (MULTI && nxt_f < p + 32) {  // ranges without a valid tuple (~0) never enter
            if (nxt_f >= p) {
                fmask |= 1u << (nxt_f - p);
                if ((uint64_t)lane == nxt_f - p) my_t = nf;
            }
            do {
                nxt_f = ++nf < c.T ? c.first_valid[nf] : ~0ull;
            } while (nf < c.T && nxt_f == ~0ull);
        }
        uint64_t pk = __shfl_up_sync(FULLW, km, 1);
        if (lane == 0) pk = prev_km;
        const bool head = valid && (i == 0 || km != pk || ((smask >> lane) & 1u));  // smask: MULTI only
        const uint32_t H = __ballot_sync(FULLW, head);
        prev_km = __shfl_sync(FULLW, km, 31);
        const bool nz = valid && km != 0 && !((zw >> lane) & 1u);
        const uint32_t r = nz ? rid : 0;
        const bool good = nz && !c.filtered[r];  // the 1-byte flags keep the probe L2-friendly
        const uint32_t G = __ballot_sync(FULLW, good);
        const int fh = H ? __ffs(H) - 1 : 32;
        const bool arr_end = p + 32 >= c.n;
        // anchor candidate of each lane's run in this window: first good lane of the run's lanes here
        int s = -1;
        if (H & le) s = 31 - __clz(H & le);
        const bool carried = s < 0;
        const uint32_t later = H & ~le;
        const int nh = later ? __ffs(later) - 1 : 32;
        const uint32_t runm = carried ? lane_range(0, fh) : lane_range(s, nh);
        const uint32_t gm = G & runm;
        const int fg = gm ? __ffs(gm) - 1 : -1;
        // quirk check by the lane holding a run's first good tuple when the run has no anchor yet
        uint32_t aval = r;
        bool quirk = false;
        if constexpr (MULTI) {
            if (good && lane == fg && !(carried && has_anchor) && ((fmask >> lane) & 1u) && km == c.r_kmer[my_t] &&
                c.r_ok[my_t]) {
                quirk = true;
                aval = c.r_min[my_t];
            }
        } else if (good && lane == fg && !(carried && has_anchor) && km == c.init_kmer && c.init_min_ok) {
            int lo = 0, hi = c.T - 1;  // the range holding i: the quirk is its first valid tuple's alone
            while (lo < hi) {
                const int m = (lo + hi + 1) >> 1;
                if (c.range_bounds[m] <= i) lo = m; else hi = m - 1;
            }
            if (c.first_valid[lo] == i) {
                quirk = true;
                aval = c.init_min;
            }
        }
        const uint32_t av = __shfl_sync(FULLW, aval, fg < 0 ? 0 : fg);
        const bool qk = __shfl_sync(FULLW, quirk, fg < 0 ? 0 : fg);
        bool do_union = false;
        uint32_t target = 0;
        if (good) {
            if (carried) {
                if (open) {
                    if (has_anchor) { do_union = true; target = anchor; }
                    else if (lane != fg || qk) { do_union = true; target = av; }
                }
            } else if (owned) {
                if (lane != fg || qk) { do_union = true; target = av; }
            }
        }
        if (do_union && target != r) uf_union(c.parent, target, r, c.err, c.uf_cap);
        // carried run bookkeeping
        if (open) {
            if (!has_anchor) {
                const uint32_t g0 = G & lane_range(0, fh);
                if (g0) { has_anchor = true; anchor = __shfl_sync(FULLW, aval, __ffs(g0) - 1); }
            }
            if (fh < 32 || arr_end) open = false;
        }
        if (!owned) continue;
        const int lh = H ? 31 - __clz(H) : -1;
        if (lh >= 0 && !arr_end) {
            const uint32_t g = G & lane_range(lh, 32);
            has_anchor = g != 0;
            anchor = has_anchor ? __shfl_sync(FULLW, aval, __ffs(g) - 1) : 0;
            open = true;
        }
    }
}

// printStats compression (metapart.c:3248-3262): every non-BAD read points at its root,
// where a BAD parent also stops the walk (unionfind.h:25-32).
__global__ void k_compress(uint32_t *parent, uint64_t n)
{
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint32_t p = parent[x];
    if (p == BAD || p == x) return;
    uint32_t y = p;
    for (uint32_t it = 0; it < UF_CAP; it++) {
        const uint32_t q = parent[y];
        if (q == y || q == BAD) break;
        y = q;
    }
    parent[x] = y;
}

// compSizes after a reset to 1 and printStats (metapart.c:4010-4030): 1 + non-root members.
// Component sizes (1 + members below each root).  The reads of a large component meet in most warps,
// so the lanes of one root add together: one atomic per root and warp instead of one per read.
__global__ void k_sizes(const uint32_t *parent, uint64_t n, uint32_t *size)
{
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t r = 0xFFFFFFFFu;
    if (x < n) {
        const uint32_t p = parent[x];
        r = (p == BAD || p == x) ? (uint32_t)x : p;
    }
    const uint32_t peers = __match_any_sync(FULLW, r);
    if (x < n && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&size[r], (uint32_t)__popc(peers));
}

// -------------------------------------------------------------- K6 mate union

// unionFindPeReads(1000) (metapart.c:2801-2867) in rounds with the same outcome as the
// reference's in-order loop.  A pair whose two roots are one is a no-op forever; a pair of
// two components above the size limit never merges (sizes only grow).  Any other pair
// depends on earlier pairs only through the small (<= limit) roots it touches, so in each
// round a pair commits when it is the earliest remaining pair on each of its small roots;
// large roots are shared: merging small components into a large one commutes.
__global__ void k_pe_prepare(uint32_t *parent, uint64_t n, uint32_t *active, uint64_t npairs)
{
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n && parent[x] == BAD) parent[x] = (uint32_t)x;  // a BAD read acts as its own root
    if (x < npairs) active[x] = (uint32_t)x;
}

__device__ __forceinline__ unsigned long long resv_key(uint32_t round, uint32_t j)
{
    return ((unsigned long long)round << 32) | (0xFFFFFFFFu - j);
}

// The round kernels read their list lengths from device memory (written by the previous kernel),
// so the host launches several rounds between synchronisations; grid-stride loops cover any length.
// The loops step whole warps (lanes past the list end idle), so a warp appends its entries to a list
// with one atomic (the order of a list's entries does not matter: a commit is decided by the round's
// reservations, not by list position).

// Appends v (where pred) to list; all 32 lanes call it.
__device__ __forceinline__ void warp_append(uint32_t *list, unsigned int *count, bool pred, uint32_t v, int lane)
{
    const uint32_t m = __ballot_sync(FULLW, pred);
    uint32_t base = 0;
    if (lane == 0 && m) base = atomicAdd(count, (unsigned int)__popc(m));
    base = __shfl_sync(FULLW, base, 0);
    if (pred) list[base + __popc(m & ((1u << lane) - 1))] = v;
}

__global__ void k_pe_reserve(uint32_t *parent, const uint32_t *size, const uint32_t *act, const unsigned int *nact_p,
                             uint32_t *act2, unsigned int *nact2, uint32_t *pra, uint32_t *prb, uint32_t *psa,
                             uint32_t *psb, unsigned long long *resv, uint32_t round, uint32_t limit)
{
    const uint32_t nact = *nact_p;
    const int lane = threadIdx.x & 31;
    for (uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < nact; w0 += gridDim.x * blockDim.x) {
        const uint32_t t = w0 + lane;
        bool keep = false, sa = false, sb = false;
        uint32_t j = 0, ra = 0, rb = 0;
        if (t < nact) {
            j = act[t];
            ra = 2 * j;
            rb = 2 * j + 1;
            uf_find2(parent, ra, rb);
            if (ra != rb) {
                const uint32_t za = size[ra], zb = size[rb];
                sa = za <= limit;
                sb = zb <= limit;
                keep = sa || sb;
                if (keep) {
                    pra[j] = ra;
                    prb[j] = rb;
                    psa[j] = za;  // sizes at the start of the round: the commit kernel changes sizes while it runs
                    psb[j] = zb;
                }
            }
        }
        warp_append(act2, nact2, keep, j, lane);
        if (keep) {
            const unsigned long long key = resv_key(round, j);
            if (sa) atomicMax(&resv[ra], key);
            if (sb) atomicMax(&resv[rb], key);
        }
    }
}

// The commit of pair j: 0 = committed a small-small merge, 1 = back to the next round's list,
// 2 = a small root under a large one (to k_pe_bigsmall).
__device__ __forceinline__ int pe_commit_one(uint32_t *parent, uint32_t *size, uint32_t j, uint32_t *pra, uint32_t *prb,
                                             const uint32_t *psa, const uint32_t *psb, const unsigned long long *resv,
                                             unsigned long long *gmax, unsigned long long *gadd, uint32_t round,
                                             uint32_t limit)
{
    const uint32_t ra = pra[j], rb = prb[j];
    const uint32_t za = psa[j], zb = psb[j];
    const bool sa = za <= limit, sb = zb <= limit;
    const unsigned long long key = resv_key(round, j);
    const bool own = (!sa || resv[ra] == key) && (!sb || resv[rb] == key);
    if (!own) return 1;
    if (sa && sb) {
        const uint32_t hi = ra > rb ? ra : rb, lo = ra > rb ? rb : ra;
        parent[lo] = hi;
        size[hi] = za + zb;
        size[lo] = 0;
        return 0;
    }
    const uint32_t g = sa ? rb : ra, x = sa ? ra : rb;
    atomicMax(&gmax[g], ((unsigned long long)round << 32) | x);
    atomicAdd(&gadd[g], (unsigned long long)(sa ? za : zb));
    pra[j] = g;  // k_pe_bigsmall reads the roles from here: sizes change while it runs
    prb[j] = x;
    return 2;
}

__global__ void k_pe_commit(uint32_t *parent, uint32_t *size, const uint32_t *act, const unsigned int *nact_p, uint32_t *next,
                            unsigned int *nnext, uint32_t *pra, uint32_t *prb, const uint32_t *psa,
                            const uint32_t *psb, const unsigned long long *resv, unsigned long long *gmax, unsigned long long *gadd,
                            uint32_t *bigsmall, unsigned int *nbig, uint32_t round, uint32_t limit)
{
    const uint32_t nact = *nact_p;
    const int lane = threadIdx.x & 31;
    for (uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < nact; w0 += gridDim.x * blockDim.x) {
        const uint32_t t = w0 + lane;
        int r = -1;
        uint32_t j = 0;
        if (t < nact) {
            j = act[t];
            r = pe_commit_one(parent, size, j, pra, prb, psa, psb, resv, gmax, gadd, round, limit);
        }
        warp_append(next, nnext, r == 1, j, lane);
        warp_append(bigsmall, nbig, r == 2, j, lane);
    }
}

__device__ __forceinline__ void pe_bigsmall_one(uint32_t *parent, uint32_t *size, uint32_t j, const uint32_t *pra,
                                                const uint32_t *prb, const unsigned long long *gmax,
                                                unsigned long long *gadd)
{
    const uint32_t g = pra[j], x = prb[j];
    const uint32_t mx = (uint32_t)(gmax[g] & 0xFFFFFFFFu);
    const uint32_t R = mx > g ? mx : g;
    if (x != mx) {  // not the designated pair of g
        parent[x] = R;
        size[x] = 0;
        return;
    }
    // designated pair (largest small root of g this round): finish the merge of g's group
    const uint32_t tot = size[g] + (uint32_t)gadd[g];
    if (R != g) {  // x is the new root
        parent[g] = R;
        size[g] = 0;
    } else {       // g stays the root: x goes under it like the others
        parent[x] = R;
        size[x] = 0;
    }
    size[R] = tot;
    gadd[g] = 0;
}

__global__ void k_pe_bigsmall(uint32_t *parent, uint32_t *size, const uint32_t *list, const unsigned int *nl_p,
                              const uint32_t *pra, const uint32_t *prb, const unsigned long long *gmax, unsigned long long *gadd)
{
    const uint32_t nl = *nl_p;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nl; t += gridDim.x * blockDim.x)
        pe_bigsmall_one(parent, size, list[t], pra, prb, gmax, gadd);
}

// --------------------------------------------------------------- host side

static unsigned blocks_for(uint64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int filter_scan(Tuples &tp, const std::vector<uint64_t> &range_bounds, uint32_t *parent, uint8_t *filtered,
                DeviceArena &arena, cudaStream_t st, bool apply_zero, bool multi)
{
    const uint64_t n = tp.n;
    const int T = (int)range_bounds.size() - 1;
    tp.z = arena.alloc<uint32_t>((n + 31) / 32 + 1);
    uint64_t *ends = arena.alloc<uint64_t>(T);
    if (!tp.z || !ends) return set_error(MP_ENOMEM, "device memory for the filter");
    MP_CUDA(cudaMemsetAsync(tp.z, 0, ((n + 31) / 32 + 1) * sizeof(uint32_t), st));
    if (n == 0) return 0;
    MP_CUDA(cudaMemcpyAsync(ends, range_bounds.data() + 1, T * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    const uint64_t warps = (n + SEG - 1) / SEG;
    if (multi)
        (mp::count_launch(), k_filter_warp<true><<<blocks_for(warps * 32, 256), 256, 0, st>>>(tp.lo, tp.hi, tp.id, n, ends, T,
                                                                                         parent, filtered, tp.z));
    else
        (mp::count_launch(), k_filter_warp<false><<<blocks_for(warps * 32, 256), 256, 0, st>>>(tp.lo, tp.hi, tp.id, n, ends, T,
                                                                                          parent, filtered, tp.z));
    if (apply_zero) (mp::count_launch(), k_apply_zero<<<blocks_for(n, 256), 256, 0, st>>>(tp.lo, tp.hi, n, tp.z));
    MP_CUDA(cudaGetLastError());
    return 0;
}

int union_scan(Tuples &tp, const std::vector<uint64_t> &range_bounds, uint32_t *parent, const uint8_t *filtered,
               uint64_t n_reads, DeviceArena &arena, cudaStream_t st, uint32_t rebad, uint32_t *hooked)
{
    const uint64_t n = tp.n;
    const int T = (int)range_bounds.size() - 1;
    *hooked = ~0u;
    uint32_t *err = arena.alloc<uint32_t>(3);  // error flags, the anchor run's read, the hooked read
    if (!err) return set_error(MP_ENOMEM, "device memory");
    MP_CUDA(cudaMemsetAsync(err, 0, 4, st));
    MP_CUDA(cudaMemsetAsync(err + 1, 0xFF, 8, st));
    if (rebad != ~0u) (mp::count_launch(), k_rebad<<<1, 1, 0, st>>>(parent, rebad));
    if (n) {
        uint64_t *bounds = arena.alloc<uint64_t>(T + 1), *first = arena.alloc<uint64_t>(T);
        if (!bounds || !first) return set_error(MP_ENOMEM, "device memory for union-find");
        MP_CUDA(cudaMemcpyAsync(bounds, range_bounds.data(), (T + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        // initial state of every range sweep: the last tuple's k-mer after the filter, the first tuple's read
        uint64_t last_lo = 0;
        uint8_t last_hi = 0;
        uint32_t zw = 0, first_id = 0;
        MP_CUDA(cudaMemcpyAsync(&last_lo, tp.lo + (n - 1), 8, cudaMemcpyDeviceToHost, st));
        if (tp.hi) MP_CUDA(cudaMemcpyAsync(&last_hi, tp.hi + (n - 1), 1, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(&zw, tp.z + ((n - 1) >> 5), 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(&first_id, tp.id, 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        uint32_t first_parent = 0;
        MP_CUDA(cudaMemcpyAsync(&first_parent, parent + first_id, 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        EdgeCtx c;
        c.lo = tp.lo; c.hi = tp.hi; c.id = tp.id; c.z = tp.z; c.n = n;
        c.first_valid = first; c.range_bounds = bounds; c.T = T; c.parent = parent; c.filtered = filtered; c.err = err;
        c.init_kmer = ((zw >> ((n - 1) & 31)) & 1u) ? 0 : ((last_lo >> 8) | ((uint64_t)last_hi << 56));
        c.init_min = first_id;
        c.init_min_ok = first_parent != BAD;
        c.r_kmer = nullptr;
        c.r_min = nullptr;
        c.r_ok = nullptr;
        c.uf_cap = arena.lim.union_retries;
        (mp::count_launch(), k_range_first_valid<<<blocks_for(T, 64), 64, 0, st>>>(tp.lo, tp.hi, tp.id, tp.z, bounds, T, parent,
                                                                                  first));
        if (!c.init_min_ok)
            (mp::count_launch(), k_bad_anchor_find<<<blocks_for(T, 64), 64, 0, st>>>(tp.lo, tp.hi, tp.id, first, T, c.init_kmer,
                                                                                    err + 1));
        const uint64_t warps = (n + SEG - 1) / SEG;
        (mp::count_launch(), k_edges_warp<false><<<blocks_for(warps * 32, 256), 256, 0, st>>>(c));
        if (!c.init_min_ok) (mp::count_launch(), k_bad_anchor_hook<<<1, 1, 0, st>>>(parent, c.init_min, err + 1, err + 2));
    }
    (mp::count_launch(), k_compress<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads));
    uint32_t h[3] = {0, 0, 0};
    MP_CUDA(cudaMemcpyAsync(h, err, sizeof h, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (h[0]) return set_error(MP_EDEVICE, "union-find retry limit reached (flags 0x%x)", h[0]);
    *hooked = h[2];
    return 0;
}

int union_piece(Tuples &tp, const std::vector<uint64_t> &bounds, const std::vector<uint8_t> &seen, uint64_t init_kmer,
                uint32_t init_min, bool init_min_ok, uint32_t *parent, const uint8_t *filtered, DeviceArena &arena,
                cudaStream_t st, std::vector<uint8_t> &has_valid, uint32_t *anchor_v)
{
    const uint64_t n = tp.n;
    const int T = (int)bounds.size() - 1;
    has_valid.assign(T, 0);
    if (n == 0 || T < 1) return 0;
    uint32_t *err = arena.alloc<uint32_t>(1);
    uint64_t *d_bounds = arena.alloc<uint64_t>(T + 1), *first = arena.alloc<uint64_t>(T);
    if (!err || !d_bounds || !first) return set_error(MP_ENOMEM, "device memory for union-find");
    MP_CUDA(cudaMemsetAsync(err, 0, sizeof *err, st));
    MP_CUDA(cudaMemcpyAsync(d_bounds, bounds.data(), (T + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    (mp::count_launch(), k_range_first_valid<<<blocks_for(T, 64), 64, 0, st>>>(tp.lo, tp.hi, tp.id, tp.z, d_bounds, T, parent,
                                                                              first));
    // a range whose first valid tuple lies in an earlier piece has none here: the quirk is that tuple's alone
    std::vector<uint64_t> hf(T);
    MP_CUDA(cudaMemcpyAsync(hf.data(), first, T * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    for (int t = 0; t < T; t++) {
        has_valid[t] = hf[t] != ~0ull;
        if (seen[t]) hf[t] = ~0ull;
    }
    MP_CUDA(cudaMemcpyAsync(first, hf.data(), T * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    if (!init_min_ok)
        (mp::count_launch(), k_bad_anchor_find<<<blocks_for(T, 64), 64, 0, st>>>(tp.lo, tp.hi, tp.id, first, T, init_kmer,
                                                                                anchor_v));
    EdgeCtx c;
    c.lo = tp.lo; c.hi = tp.hi; c.id = tp.id; c.z = tp.z; c.n = n;
    c.first_valid = first; c.range_bounds = d_bounds; c.T = T; c.parent = parent; c.filtered = filtered; c.err = err;
    c.init_kmer = init_kmer;
    c.init_min = init_min;
    c.init_min_ok = init_min_ok ? 1u : 0u;
    c.r_kmer = nullptr;
    c.r_min = nullptr;
    c.r_ok = nullptr;
    c.uf_cap = arena.lim.union_retries;
    const uint64_t warps = (n + SEG - 1) / SEG;
    (mp::count_launch(), k_edges_warp<false><<<blocks_for(warps * 32, 256), 256, 0, st>>>(c));
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (herr) return set_error(MP_EDEVICE, "union-find retry limit reached (flags 0x%x)", herr);
    return 0;
}

// Reads whose parent is neither BAD nor a root (its own parent): none after a compression.
__global__ void k_count_nonroot(const uint32_t *parent, uint64_t n, unsigned long long *out)
{
    unsigned long long c = 0;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t p = parent[x];
        c += (p != BAD && (p >= n || parent[p] != p)) ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(FULLW, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

int count_nonroot(const uint32_t *parent, uint64_t n, unsigned long long *d_count, cudaStream_t st, uint64_t *out)
{
    MP_CUDA(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    if (n) {
        const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, 8ull * (uint64_t)sm_count());
        (mp::count_launch(), k_count_nonroot<<<(unsigned)blocks, 256, 0, st>>>(parent, n, d_count));
    }
    unsigned long long h = 0;
    MP_CUDA(cudaMemcpyAsync(&h, d_count, sizeof h, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    *out = h;
    return 0;
}

void rebad_read(uint32_t *parent, uint32_t r, cudaStream_t st)
{
    if (r != ~0u) (mp::count_launch(), k_rebad<<<1, 1, 0, st>>>(parent, r));
}

void hook_bad_anchor(uint32_t *parent, uint32_t b, const uint32_t *anchor_v, uint32_t *hooked, cudaStream_t st)
{
    (mp::count_launch(), k_bad_anchor_hook<<<1, 1, 0, st>>>(parent, b, anchor_v, hooked));
}

void compress_parents(uint32_t *parent, uint64_t n_reads, cudaStream_t st)
{
    (mp::count_launch(), k_compress<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads));
}

int mate_union_and_plan(uint32_t *parent, uint64_t n_reads, uint32_t *size, uint64_t *bounds_out, DeviceArena &arena,
                        cudaStream_t st, int *rounds_out)
{
    int rc = mate_union(parent, n_reads, size, arena, st, rounds_out);
    return rc ? rc : plan_partitions(parent, size, n_reads, bounds_out, arena, st);
}

int mate_union(uint32_t *parent, uint64_t n_reads, uint32_t *size, DeviceArena &arena, cudaStream_t st, int *rounds_out)
{
    const uint32_t limit = 1000;
    const uint64_t npairs = n_reads / 2;
    MP_CUDA(cudaMemsetAsync(size, 0, n_reads * sizeof(uint32_t), st));
    (mp::count_launch(), k_sizes<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads, size));
    uint32_t *act = arena.alloc<uint32_t>(npairs + 1), *act2 = arena.alloc<uint32_t>(npairs + 1);
    uint32_t *pra = arena.alloc<uint32_t>(npairs + 1), *prb = arena.alloc<uint32_t>(npairs + 1);
    uint32_t *big = arena.alloc<uint32_t>(npairs + 1);
    uint32_t *psa = arena.alloc<uint32_t>(npairs + 1), *psb = arena.alloc<uint32_t>(npairs + 1);
    unsigned long long *resv = arena.alloc<unsigned long long>(n_reads);
    unsigned long long *gmax = arena.alloc<unsigned long long>(n_reads);
    unsigned long long *gadd = arena.alloc<unsigned long long>(n_reads);
    constexpr int RB = 8;  // rounds launched between host synchronisations
    // per round r of a batch: [4r] reserved pairs, [4r+1] pairs left for the next round, [4r+2] big-small merges;
    // [4 RB + 1] the batch's first active count
    unsigned int *cnts = arena.alloc<unsigned int>(4 * RB + 4);
    if (!act || !act2 || !pra || !prb || !big || !psa || !psb || !resv || !gmax || !gadd || !cnts)
        return set_error(MP_ENOMEM, "device memory for the mate union");
    MP_CUDA(cudaMemsetAsync(resv, 0, n_reads * sizeof(unsigned long long), st));
    MP_CUDA(cudaMemsetAsync(gmax, 0, n_reads * sizeof(unsigned long long), st));
    MP_CUDA(cudaMemsetAsync(gadd, 0, n_reads * sizeof(unsigned long long), st));
    (mp::count_launch(), k_pe_prepare<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads, act, npairs));
    uint32_t nact = (uint32_t)npairs, round = 0;
    while (nact > 0) {
        if (round + RB > arena.lim.mate_rounds)
            return set_error(MP_EDEVICE, "mate union did not converge within %u rounds", arena.lim.mate_rounds);
        // counts only shrink, so nact bounds every list of the batch
        const unsigned g = (unsigned)std::min<uint64_t>(blocks_for(nact, 256), 8ull * (uint64_t)sm_count());
        MP_CUDA(cudaMemsetAsync(cnts, 0, (4 * RB + 4) * sizeof(unsigned int), st));
        MP_CUDA(cudaMemcpyAsync(cnts + 4 * RB + 1, &nact, sizeof(unsigned int), cudaMemcpyHostToDevice, st));
        for (int r = 0; r < RB; r++) {
            ++round;
            const unsigned int *nin = r ? cnts + 4 * (r - 1) + 1 : cnts + 4 * RB + 1;
            (mp::count_launch(), k_pe_reserve<<<g, 256, 0, st>>>(parent, size, act, nin, act2, cnts + 4 * r, pra, prb, psa,
                                                                 psb, resv, round, limit));
            (mp::count_launch(), k_pe_commit<<<g, 256, 0, st>>>(parent, size, act2, cnts + 4 * r, act, cnts + 4 * r + 1, pra,
                                                                prb, psa, psb, resv, gmax, gadd, big, cnts + 4 * r + 2,
                                                                round, limit));
            (mp::count_launch(), k_pe_bigsmall<<<g, 256, 0, st>>>(parent, size, big, cnts + 4 * r + 2, pra, prb, gmax, gadd));
        }
        unsigned int h[4 * RB + 4];
        MP_CUDA(cudaMemcpyAsync(h, cnts, sizeof h, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        nact = h[4 * (RB - 1) + 1];
        // rounds that reserved nothing leave nothing active: stop counting at the first empty one
        for (int r = 0; r < RB; r++)
            if (h[4 * r] == 0) {
                round -= (uint32_t)(RB - 1 - r);
                nact = 0;
                break;
            }
    }
    if (rounds_out) *rounds_out = (int)round;
    // final printStats: compress and recount (metapart.c:4026-4030)
    (mp::count_launch(), k_compress<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads));
    MP_CUDA(cudaMemsetAsync(size, 0, n_reads * sizeof(uint32_t), st));
    (mp::count_launch(), k_sizes<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads, size));
    return 0;
}

// Work partitions (metapart.c:4036-4053): bound i = first read id c at which the sizes of
// the roots below c reach i * floor(N / 16).
__global__ void k_root_weight(const uint32_t *parent, const uint32_t *size, uint64_t n, uint32_t *w)
{
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) w[x] = parent[x] == x ? size[x] : 0u;
}
__global__ void k_bounds(const uint64_t *pre, uint64_t n, uint64_t *bounds)
{
    const int i = threadIdx.x;
    if (i > 16) return;
    if (i == 0) { bounds[0] = 0; return; }
    if (i == 16) { bounds[16] = n; return; }
    const uint64_t thr = (uint64_t)i * (n / 16);
    uint64_t lo = 0, hi = n;  // smallest c in [0, n] with pre[c] >= thr
    while (lo < hi) {
        uint64_t m = (lo + hi) / 2;
        if (pre[m] >= thr) hi = m; else lo = m + 1;
    }
    bounds[i] = lo;
}

int plan_partitions(const uint32_t *parent, const uint32_t *size, uint64_t n_reads, uint64_t *bounds_host,
                    DeviceArena &arena, cudaStream_t st)
{
    uint32_t *w = arena.alloc<uint32_t>(n_reads + 1);
    uint64_t *pre = arena.alloc<uint64_t>(n_reads + 1);
    uint64_t *b = arena.alloc<uint64_t>(17);
    size_t tb = scan_tmp_bytes(n_reads + 1);
    void *tmp = arena.alloc<uint8_t>(tb);
    if (!w || !pre || !b || !tmp) return set_error(MP_ENOMEM, "device memory for the partition planner");
    MP_CUDA(cudaMemsetAsync(w + n_reads, 0, sizeof(uint32_t), st));
    (mp::count_launch(), k_root_weight<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, size, n_reads, w));
    scan_u32_to_u64(w, pre, n_reads + 1, nullptr, tmp, tb, st);
    (mp::count_launch(), k_bounds<<<1, 32, 0, st>>>(pre, n_reads, b));
    MP_CUDA(cudaMemcpyAsync(bounds_host, b, 17 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    return 0;
}

// ------------------------------------------------------ batches of samples

// The initial sweep state of every thread range of a batch: its sample's scan's last k-mer (after the
// filter's zero marks), first read, and whether that read is BAD as the unions begin (metapart.c:2539-2548).
__global__ void k_seg_union_init(const uint64_t *lo, const uint8_t *hi, const uint32_t *id, const uint32_t *z,
                                 const uint64_t *seg_tstart, const uint32_t *range_seg, int nranges, const uint32_t *parent,
                                 uint64_t *r_kmer, uint32_t *r_min, uint32_t *r_ok)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nranges) return;
    const uint32_t q = range_seg[t];
    const uint64_t a = seg_tstart[q], b = seg_tstart[q + 1];
    if (a == b) {  // a sample without tuples: its ranges are empty
        r_kmer[t] = 0;
        r_min[t] = 0;
        r_ok[t] = 0;
        return;
    }
    const uint64_t last = b - 1;
    r_kmer[t] = zbit(z, last) ? 0ull : kmer_of(lo, hi, last);
    const uint32_t f = id[a];
    r_min[t] = f;
    r_ok[t] = parent[f] != BAD ? 1u : 0u;
}

int union_segments(Tuples &tp, const std::vector<uint64_t> &range_bounds, const std::vector<uint32_t> &range_seg,
                   const std::vector<uint64_t> &seg_tstart, uint32_t *parent, const uint8_t *filtered, uint64_t n_reads,
                   DeviceArena &arena, cudaStream_t st)
{
    const uint64_t n = tp.n;
    const int R = (int)range_bounds.size() - 1, nseg = (int)seg_tstart.size() - 1;
    uint32_t *err = arena.alloc<uint32_t>(1);
    if (!err) return set_error(MP_ENOMEM, "device memory");
    MP_CUDA(cudaMemsetAsync(err, 0, sizeof *err, st));
    if (n) {
        uint64_t *bounds = arena.alloc<uint64_t>(R + 1), *first = arena.alloc<uint64_t>(R), *ts = arena.alloc<uint64_t>(nseg + 1);
        uint64_t *rk = arena.alloc<uint64_t>(R);
        uint32_t *rs = arena.alloc<uint32_t>(R), *rm = arena.alloc<uint32_t>(R), *ro = arena.alloc<uint32_t>(R);
        if (!bounds || !first || !ts || !rk || !rs || !rm || !ro) return set_error(MP_ENOMEM, "device memory for union-find");
        MP_CUDA(cudaMemcpyAsync(bounds, range_bounds.data(), (R + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        MP_CUDA(cudaMemcpyAsync(rs, range_seg.data(), R * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        MP_CUDA(cudaMemcpyAsync(ts, seg_tstart.data(), (nseg + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        (mp::count_launch(), k_seg_union_init<<<blocks_for(R, 128), 128, 0, st>>>(tp.lo, tp.hi, tp.id, tp.z, ts, rs, R, parent,
                                                                                 rk, rm, ro));
        (mp::count_launch(), k_range_first_valid<<<blocks_for(R, 64), 64, 0, st>>>(tp.lo, tp.hi, tp.id, tp.z, bounds, R, parent,
                                                                                  first));
        EdgeCtx c;
        c.lo = tp.lo; c.hi = tp.hi; c.id = tp.id; c.z = tp.z; c.n = n;
        c.first_valid = first; c.range_bounds = bounds; c.T = R; c.parent = parent; c.filtered = filtered; c.err = err;
        c.init_kmer = 0;
        c.init_min = 0;
        c.init_min_ok = 0;
        c.r_kmer = rk;
        c.r_min = rm;
        c.r_ok = ro;
        c.uf_cap = arena.lim.union_retries;
        const uint64_t warps = (n + SEG - 1) / SEG;
        (mp::count_launch(), k_edges_warp<true><<<blocks_for(warps * 32, 256), 256, 0, st>>>(c));
        (mp::count_launch(), k_seg_bad_anchor<<<blocks_for(R, 64), 64, 0, st>>>(tp.lo, tp.hi, tp.id, first, R, rk, rm, ro, parent));
    }
    (mp::count_launch(), k_compress<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads));
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (herr) return set_error(MP_EDEVICE, "union-find retry limit reached (flags 0x%x)", herr);
    return 0;
}

// The 16 work partitions of every sample of a batch (metapart.c:4036-4053 per sample): bounds in the
// sample's own read ids, from the prefix of root weights over all reads.
__global__ void k_seg_bounds(const uint64_t *pre, const uint64_t *srec, int nseg, uint64_t *bounds)
{
    const int q = blockIdx.x, i = threadIdx.x;
    if (q >= nseg || i > 16) return;
    const uint64_t R = srec[q], N = srec[q + 1] - R;
    uint64_t *b = bounds + (uint64_t)q * 17;
    if (i == 0) { b[0] = 0; return; }
    if (i == 16) { b[16] = N; return; }
    const uint64_t thr = (uint64_t)i * (N / 16), base = pre[R];
    uint64_t lo = 0, hi = N;  // smallest c in [0, N] with the weights of reads R .. R + c - 1 reaching thr
    while (lo < hi) {
        const uint64_t m = (lo + hi) / 2;
        if (pre[R + m] - base >= thr) hi = m; else lo = m + 1;
    }
    b[i] = lo;
}

int plan_partitions_segments(const uint32_t *parent, const uint32_t *size, uint64_t n_reads,
                             const std::vector<uint64_t> &seg_reads, uint64_t *bounds_host, DeviceArena &arena,
                             cudaStream_t st)
{
    const int nseg = (int)seg_reads.size() - 1;
    uint32_t *w = arena.alloc<uint32_t>(n_reads + 1);
    uint64_t *pre = arena.alloc<uint64_t>(n_reads + 1), *srec = arena.alloc<uint64_t>(nseg + 1);
    uint64_t *b = arena.alloc<uint64_t>((size_t)nseg * 17);
    size_t tb = scan_tmp_bytes(n_reads + 1);
    void *tmp = arena.alloc<uint8_t>(tb);
    if (!w || !pre || !srec || !b || !tmp) return set_error(MP_ENOMEM, "device memory for the partition planner");
    MP_CUDA(cudaMemsetAsync(w + n_reads, 0, sizeof(uint32_t), st));
    MP_CUDA(cudaMemcpyAsync(srec, seg_reads.data(), (nseg + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    (mp::count_launch(), k_root_weight<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, size, n_reads, w));
    scan_u32_to_u64(w, pre, n_reads + 1, nullptr, tmp, tb, st);
    (mp::count_launch(), k_seg_bounds<<<nseg, 32, 0, st>>>(pre, srec, nseg, b));
    MP_CUDA(cudaMemcpyAsync(bounds_host, b, (size_t)nseg * 17 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace mp
