// K4 (branching k-mer filter), K5 (run edges + union-find), K6 (mate union) and the
// partition planner, on the sorted tuples of one scan and the per-read parent array.
//
// parent[] is the reference's parent array as u32 with BAD = 0xFFFFFFFF standing for
// 0xBADBADBAD (metapart.c:2330-2340).  Components hook the smaller root under the larger
// one, so every component's root is its largest read id (metapart.c:2683-2716,
// unionfind.h:58-66) regardless of the order unions run in.
#include <vector>

#include "k_graph.cuh"

namespace mp {

constexpr int LONG_RUN = 256;    // runs longer than this go to the block-per-run kernels
constexpr uint32_t UF_CAP = 1u << 20;

__device__ __forceinline__ uint64_t kmer_of(const uint64_t *lo, const uint8_t *hi, uint64_t i)
{
    return (lo[i] >> 8) | (hi ? ((uint64_t)hi[i] << 56) : 0ull);
}

// ----------------------------------------------------------------- runs

__global__ void k_run_heads(const uint64_t *lo, const uint8_t *hi, uint64_t n, uint32_t *heads)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool h = i < n && (i == 0 || kmer_of(lo, hi, i) != kmer_of(lo, hi, i - 1));
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, h);
    if ((threadIdx.x & 31) == 0 && i < n + 31) heads[i >> 5] = b;
}

// end of the run starting at s: the next head after s (or n)
__device__ __forceinline__ uint64_t run_end(const uint32_t *heads, uint64_t n, uint64_t s)
{
    uint64_t i = s + 1;
    if (i >= n) return n;
    uint64_t w = i >> 5;
    uint32_t m = heads[w] & (0xFFFFFFFFu << (i & 31));
    const uint64_t nw = (n + 31) >> 5;
    while (!m) {
        if (++w >= nw) return n;
        m = heads[w];
    }
    const uint64_t e = (w << 5) + (uint64_t)(__ffs(m) - 1);
    return e < n ? e : n;
}

__device__ __forceinline__ bool is_head(const uint32_t *heads, uint64_t i) { return (heads[i >> 5] >> (i & 31)) & 1u; }

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

// --------------------------------------------------------------- K4 filter

struct Judge {
    int nin, nout, mxi, mxo;
    bool zero, ratio_bad;
};

// markMischiefKmers decision for one run (metapart.c:2296-2451)
__device__ __forceinline__ Judge judge_run(const uint32_t *before, const uint32_t *after, uint32_t deg)
{
    Judge j{0, 0, 0, 0, false, false};
    uint32_t cmi = 0, cmo = 0, smi = 0, smo = 0;
    for (int q = 0; q < 7; q++) {
        if (before[q]) {
            if (before[q] > cmi) { smi = cmi; cmi = before[q]; j.mxi = q; }
            else if (before[q] > smi) smi = before[q];
            j.nin++;
        }
        if (after[q]) {
            if (after[q] > cmo) { smo = cmo; cmo = after[q]; j.mxo = q; }
            else if (after[q] > smo) smo = after[q];
            j.nout++;
        }
    }
    j.zero = j.nin > 1 && j.nout > 1;
    // (float)count / degree compared with 0.2 as double, as the reference does
    const float r_in = __fdiv_rn((float)smi, (float)deg), r_out = __fdiv_rn((float)smo, (float)deg);
    j.ratio_bad = ((double)r_in > 0.2) || ((double)r_out > 0.2);
    return j;
}

__device__ __forceinline__ void apply_marks(const Judge &jd, uint64_t s, uint64_t e, uint64_t *lo, uint8_t *hi,
                                            const uint32_t *id, uint32_t *parent, uint8_t *filtered)
{
    for (uint64_t q = s; q < e; q++) {
        const uint32_t adj = (uint32_t)(lo[q] & 0xFF);
        if (jd.zero) {
            lo[q] = adj;
            if (hi) hi[q] = 0;
            continue;
        }
        const uint32_t bi = adj & 7, ai = (adj >> 3) & 7;
        bool bad = (jd.nin > 1 && bi != (uint32_t)jd.mxi) || (jd.nout > 1 && ai != (uint32_t)jd.mxo);
        if (!bad) bad = jd.ratio_bad;
        if (bad) {
            const uint32_t r = id[q];
            parent[r] = BAD;
            filtered[r] = 1;
        }
    }
}

__global__ void k_filter(uint64_t *lo, uint8_t *hi, const uint32_t *id, uint64_t n, const uint32_t *heads,
                         const uint64_t *range_ends, int T, uint32_t *parent, uint8_t *filtered, uint64_t *long_runs,
                         unsigned long long *n_long)
{
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || !is_head(heads, s)) return;
    const uint64_t e = run_end(heads, n, s);
    if (at_range_end(range_ends, T, e)) return;
    if (e - s > (uint64_t)LONG_RUN) {
        long_runs[atomicAdd(n_long, 1ull)] = s;
        return;
    }
    uint32_t before[8] = {0}, after[8] = {0};
    for (uint64_t q = s; q < e; q++) {
        const uint32_t adj = (uint32_t)(lo[q] & 0xFF);
        before[adj & 7]++;
        after[(adj >> 3) & 7]++;
    }
    const Judge jd = judge_run(before, after, (uint32_t)(e - s));
    if (jd.nin > 1 || jd.nout > 1) apply_marks(jd, s, e, lo, hi, id, parent, filtered);
}

__global__ void k_filter_long(uint64_t *lo, uint8_t *hi, const uint32_t *id, uint64_t n, const uint32_t *heads,
                              const uint64_t *long_runs, uint32_t *parent, uint8_t *filtered)
{
    __shared__ uint32_t cnt[16];
    __shared__ Judge jd;
    const uint64_t s = long_runs[blockIdx.x];
    const uint64_t e = run_end(heads, n, s);
    if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
    __syncthreads();
    uint32_t b[8] = {0}, a[8] = {0};
    for (uint64_t q = s + threadIdx.x; q < e; q += blockDim.x) {
        const uint32_t adj = (uint32_t)(lo[q] & 0xFF);
        b[adj & 7]++;
        a[(adj >> 3) & 7]++;
    }
    for (int x = 0; x < 8; x++) {
        if (b[x]) atomicAdd(&cnt[x], b[x]);
        if (a[x]) atomicAdd(&cnt[8 + x], a[x]);
    }
    __syncthreads();
    if (threadIdx.x == 0) jd = judge_run(cnt, cnt + 8, (uint32_t)(e - s));
    __syncthreads();
    if (!(jd.nin > 1 || jd.nout > 1)) return;
    for (uint64_t q = s + threadIdx.x; q < e; q += blockDim.x) apply_marks(jd, q, q + 1, lo, hi, id, parent, filtered);
}

// ---------------------------------------------------------- union-find

__device__ __forceinline__ uint32_t uf_find(uint32_t *parent, uint32_t x)
{
    uint32_t p = parent[x];
    while (p != x && p != BAD) {
        const uint32_t gp = parent[p];
        if (gp == p || gp == BAD) return p;
        parent[x] = gp;  // path halving: gp is an ancestor of x
        x = gp;
        p = parent[x];
    }
    return x;
}

__device__ __forceinline__ void uf_union(uint32_t *parent, uint32_t a, uint32_t b, uint32_t *err)
{
    for (uint32_t it = 0; it < UF_CAP; it++) {
        const uint32_t ra = uf_find(parent, a), rb = uf_find(parent, b);
        if (ra == rb) return;
        const uint32_t hi = ra > rb ? ra : rb, lo = ra > rb ? rb : ra;
        if (atomicCAS(&parent[lo], lo, hi) == lo) return;
    }
    atomicOr(err, DERR_SPIN);
}

// First tuple of each thread range whose k-mer is non-zero and whose read is not BAD.
__global__ void k_range_first_valid(const uint64_t *lo, const uint8_t *hi, const uint32_t *id, const uint64_t *range_bounds,
                                    int T, const uint32_t *parent, uint64_t *first)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    uint64_t f = ~0ull;
    for (uint64_t q = range_bounds[t]; q < range_bounds[t + 1]; q++)
        if (kmer_of(lo, hi, q) != 0 && parent[id[q]] != BAD) { f = q; break; }
    first[t] = f;
}

struct EdgeCtx {
    const uint64_t *lo;
    const uint8_t *hi;
    const uint32_t *id;
    uint64_t n;
    const uint32_t *heads;
    const uint64_t *first_valid;   // per thread range
    const uint64_t *range_bounds;  // T + 1 tuple bounds
    int T;
    uint64_t init_kmer;            // k-mer of the scan's last tuple (metapart.c:2541)
    uint32_t init_min;             // read id of the scan's first tuple (metapart.c:2543-2545)
    uint32_t *parent;
    uint32_t *err;
};

// Anchor of a run: the first valid tuple's read, or -- for the first valid run of a thread
// range whose k-mer equals the scan's last k-mer -- the first tuple's read (the reference
// starts every range with that state, metapart.c:2539-2548).  Returns false when the run
// yields no edges.
__device__ __forceinline__ bool run_anchor(const EdgeCtx &c, uint64_t s, uint64_t e, uint64_t &first, uint32_t &anchor,
                                           bool &quirk)
{
    const uint64_t km = kmer_of(c.lo, c.hi, s);
    if (km == 0) return false;
    uint64_t f = e;
    for (uint64_t q = s; q < e; q++)
        if (c.parent[c.id[q]] != BAD) { f = q; break; }
    if (f == e) return false;
    first = f;
    anchor = c.id[f];
    quirk = false;
    if (km == c.init_kmer) {
        int lo = 0, hi = c.T - 1;  // thread range containing s
        while (lo < hi) {
            int m = (lo + hi + 1) >> 1;
            if (c.range_bounds[m] <= s) lo = m; else hi = m - 1;
        }
        if (c.first_valid[lo] == f && c.parent[c.init_min] != BAD) {
            anchor = c.init_min;
            quirk = true;
        }
    }
    return true;
}

__global__ void k_edges(EdgeCtx c, uint64_t *long_runs, unsigned long long *n_long)
{
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= c.n || !is_head(c.heads, s)) return;
    const uint64_t e = run_end(c.heads, c.n, s);
    if (e - s > (uint64_t)LONG_RUN) {
        long_runs[atomicAdd(n_long, 1ull)] = s;
        return;
    }
    uint64_t f;
    uint32_t anchor;
    bool quirk;
    if (!run_anchor(c, s, e, f, anchor, quirk)) return;
    for (uint64_t q = quirk ? f : f + 1; q < e; q++) {
        const uint32_t r = c.id[q];
        if (r == anchor || c.parent[r] == BAD) continue;
        uf_union(c.parent, anchor, r, c.err);
    }
}

__global__ void k_edges_long(EdgeCtx c, const uint64_t *long_runs)
{
    __shared__ uint64_t sf;
    __shared__ uint32_t sa;
    __shared__ int sq, ok;
    const uint64_t s = long_runs[blockIdx.x];
    const uint64_t e = run_end(c.heads, c.n, s);
    if (threadIdx.x == 0) {
        uint64_t f;
        uint32_t a;
        bool q;
        ok = run_anchor(c, s, e, f, a, q);
        sf = f; sa = a; sq = q;
    }
    __syncthreads();
    if (!ok) return;
    for (uint64_t q = (sq ? sf : sf + 1) + threadIdx.x; q < e; q += blockDim.x) {
        const uint32_t r = c.id[q];
        if (r == sa || c.parent[r] == BAD) continue;
        uf_union(c.parent, sa, r, c.err);
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
__global__ void k_sizes(const uint32_t *parent, uint64_t n, uint32_t *size)
{
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint32_t p = parent[x];
    atomicAdd(&size[(p == BAD || p == x) ? (uint32_t)x : p], 1u);
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

__global__ void k_pe_reserve(uint32_t *parent, const uint32_t *size, const uint32_t *act, uint32_t nact,
                             uint32_t *act2, unsigned int *nact2, uint32_t *pra, uint32_t *prb, uint32_t *psa,
                             uint32_t *psb, unsigned long long *resv, uint32_t round, uint32_t limit)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nact) return;
    const uint32_t j = act[t];
    const uint32_t ra = uf_find(parent, 2 * j), rb = uf_find(parent, 2 * j + 1);
    if (ra == rb) return;
    const uint32_t za = size[ra], zb = size[rb];
    const bool sa = za <= limit, sb = zb <= limit;
    if (!sa && !sb) return;
    pra[j] = ra;
    prb[j] = rb;
    psa[j] = za;  // sizes at the start of the round: the commit kernel changes sizes while it runs
    psb[j] = zb;
    act2[atomicAdd(nact2, 1u)] = j;
    const unsigned long long key = resv_key(round, j);
    if (sa) atomicMax(&resv[ra], key);
    if (sb) atomicMax(&resv[rb], key);
}

__global__ void k_pe_commit(uint32_t *parent, uint32_t *size, const uint32_t *act, uint32_t nact, uint32_t *next,
                            unsigned int *nnext, uint32_t *pra, uint32_t *prb, const uint32_t *psa,
                            const uint32_t *psb, const unsigned long long *resv, unsigned long long *gmax, unsigned long long *gadd,
                            uint32_t *bigsmall, unsigned int *nbig, uint32_t round, uint32_t limit)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nact) return;
    const uint32_t j = act[t];
    const uint32_t ra = pra[j], rb = prb[j];
    const uint32_t za = psa[j], zb = psb[j];
    const bool sa = za <= limit, sb = zb <= limit;
    const unsigned long long key = resv_key(round, j);
    const bool own = (!sa || resv[ra] == key) && (!sb || resv[rb] == key);
    if (!own) {
        next[atomicAdd(nnext, 1u)] = j;
        return;
    }
    if (sa && sb) {
        const uint32_t hi = ra > rb ? ra : rb, lo = ra > rb ? rb : ra;
        parent[lo] = hi;
        size[hi] = za + zb;
        size[lo] = 0;
        return;
    }
    const uint32_t g = sa ? rb : ra, x = sa ? ra : rb;
    atomicMax(&gmax[g], ((unsigned long long)round << 32) | x);
    atomicAdd(&gadd[g], (unsigned long long)(sa ? za : zb));
    pra[j] = g;  // k_pe_bigsmall reads the roles from here: sizes change while it runs
    prb[j] = x;
    bigsmall[atomicAdd(nbig, 1u)] = j;
}

__global__ void k_pe_bigsmall(uint32_t *parent, uint32_t *size, const uint32_t *list, uint32_t nl, const uint32_t *pra,
                              const uint32_t *prb, const unsigned long long *gmax, unsigned long long *gadd)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl) return;
    const uint32_t j = list[t];
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

// --------------------------------------------------------------- host side

static unsigned blocks_for(uint64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int filter_scan(Tuples &tp, const std::vector<uint64_t> &range_bounds, uint32_t *parent, uint8_t *filtered,
                DeviceArena &arena, cudaStream_t st)
{
    const uint64_t n = tp.n;
    if (n == 0) return 0;
    const int T = (int)range_bounds.size() - 1;
    tp.heads = arena.alloc<uint32_t>((n + 31) / 32 + 1);
    uint64_t *ends = arena.alloc<uint64_t>(T);
    uint64_t *long_runs = arena.alloc<uint64_t>(n / LONG_RUN + 2);
    unsigned long long *nlong = arena.alloc<unsigned long long>(1);
    if (!tp.heads || !ends || !long_runs || !nlong) return set_error(MP_ENOMEM, "device memory for the filter");
    MP_CUDA(cudaMemcpyAsync(ends, range_bounds.data() + 1, T * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemsetAsync(nlong, 0, sizeof *nlong, st));
    (mp::count_launch(), k_run_heads<<<blocks_for(n, 256), 256, 0, st>>>(tp.lo, tp.hi, n, tp.heads));
    (mp::count_launch(), k_filter<<<blocks_for(n, 256), 256, 0, st>>>(tp.lo, tp.hi, tp.id, n, tp.heads, ends, T, parent, filtered,
                                                 long_runs, nlong));
    unsigned long long hl = 0;
    MP_CUDA(cudaMemcpyAsync(&hl, nlong, sizeof hl, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    if (hl) (mp::count_launch(), k_filter_long<<<(unsigned)hl, 256, 0, st>>>(tp.lo, tp.hi, tp.id, n, tp.heads, long_runs, parent, filtered));
    MP_CUDA(cudaGetLastError());
    return 0;
}

int union_scan(Tuples &tp, const std::vector<uint64_t> &range_bounds, uint32_t *parent, uint64_t n_reads,
               DeviceArena &arena, cudaStream_t st)
{
    const uint64_t n = tp.n;
    const int T = (int)range_bounds.size() - 1;
    uint32_t *err = arena.alloc<uint32_t>(1);
    if (!err) return set_error(MP_ENOMEM, "device memory");
    MP_CUDA(cudaMemsetAsync(err, 0, sizeof *err, st));
    if (n) {
        uint64_t *bounds = arena.alloc<uint64_t>(T + 1), *first = arena.alloc<uint64_t>(T);
        uint64_t *long_runs = arena.alloc<uint64_t>(n / LONG_RUN + 2);
        unsigned long long *nlong = arena.alloc<unsigned long long>(1);
        if (!bounds || !first || !long_runs || !nlong) return set_error(MP_ENOMEM, "device memory for union-find");
        MP_CUDA(cudaMemcpyAsync(bounds, range_bounds.data(), (T + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        MP_CUDA(cudaMemsetAsync(nlong, 0, sizeof *nlong, st));
        EdgeCtx c;
        c.lo = tp.lo; c.hi = tp.hi; c.id = tp.id; c.n = n; c.heads = tp.heads;
        c.first_valid = first; c.range_bounds = bounds; c.T = T; c.parent = parent; c.err = err;
        // initial state of every range sweep: last tuple's k-mer, first tuple's read (post filter)
        uint64_t last_lo = 0, id0 = 0;
        uint8_t last_hi = 0;
        uint32_t first_id = 0;
        MP_CUDA(cudaMemcpyAsync(&last_lo, tp.lo + (n - 1), 8, cudaMemcpyDeviceToHost, st));
        if (tp.hi) MP_CUDA(cudaMemcpyAsync(&last_hi, tp.hi + (n - 1), 1, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(&first_id, tp.id, 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        (void)id0;
        c.init_kmer = (last_lo >> 8) | ((uint64_t)last_hi << 56);
        c.init_min = first_id;
        (mp::count_launch(), k_range_first_valid<<<blocks_for(T, 64), 64, 0, st>>>(tp.lo, tp.hi, tp.id, bounds, T, parent, first));
        (mp::count_launch(), k_edges<<<blocks_for(n, 256), 256, 0, st>>>(c, long_runs, nlong));
        unsigned long long hl = 0;
        MP_CUDA(cudaMemcpyAsync(&hl, nlong, sizeof hl, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        if (hl) (mp::count_launch(), k_edges_long<<<(unsigned)hl, 256, 0, st>>>(c, long_runs));
    }
    (mp::count_launch(), k_compress<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads));
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (herr) return set_error(MP_EDEVICE, "union-find retry limit reached (flags 0x%x)", herr);
    return 0;
}

int mate_union_and_plan(uint32_t *parent, uint64_t n_reads, uint32_t *size, uint64_t *bounds_out, DeviceArena &arena,
                        cudaStream_t st, int *rounds_out)
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
    unsigned int *cnts = arena.alloc<unsigned int>(4);
    if (!act || !act2 || !pra || !prb || !big || !psa || !psb || !resv || !gmax || !gadd || !cnts)
        return set_error(MP_ENOMEM, "device memory for the mate union");
    MP_CUDA(cudaMemsetAsync(resv, 0, n_reads * sizeof(unsigned long long), st));
    MP_CUDA(cudaMemsetAsync(gmax, 0, n_reads * sizeof(unsigned long long), st));
    MP_CUDA(cudaMemsetAsync(gadd, 0, n_reads * sizeof(unsigned long long), st));
    (mp::count_launch(), k_pe_prepare<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads, act, npairs));
    uint32_t nact = (uint32_t)npairs, round = 0;
    while (nact > 0) {
        if (++round > 4000000u) return set_error(MP_EDEVICE, "mate union did not converge");
        MP_CUDA(cudaMemsetAsync(cnts, 0, 4 * sizeof(unsigned int), st));
        (mp::count_launch(), k_pe_reserve<<<blocks_for(nact, 256), 256, 0, st>>>(parent, size, act, nact, act2, cnts, pra, prb, psa, psb,
                                                            resv, round, limit));
        unsigned int h[3] = {0, 0, 0};
        MP_CUDA(cudaMemcpyAsync(h, cnts, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        if (h[0] == 0) break;
        (mp::count_launch(), k_pe_commit<<<blocks_for(h[0], 256), 256, 0, st>>>(parent, size, act2, h[0], act, cnts + 1, pra, prb, psa,
                                                           psb, resv, gmax, gadd, big, cnts + 2, round, limit));
        MP_CUDA(cudaMemcpyAsync(h, cnts, 3 * sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        if (h[2]) (mp::count_launch(), k_pe_bigsmall<<<blocks_for(h[2], 256), 256, 0, st>>>(parent, size, big, h[2], pra, prb, gmax, gadd));
        nact = h[1];
    }
    if (rounds_out) *rounds_out = (int)round;
    // final printStats: compress and recount (metapart.c:4026-4030)
    (mp::count_launch(), k_compress<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads));
    MP_CUDA(cudaMemsetAsync(size, 0, n_reads * sizeof(uint32_t), st));
    (mp::count_launch(), k_sizes<<<blocks_for(n_reads, 256), 256, 0, st>>>(parent, n_reads, size));
    return plan_partitions(parent, size, n_reads, bounds_out, arena, st);
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

}  // namespace mp
