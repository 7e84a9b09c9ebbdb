// K3: stable LSD radix sort of (k-mer, adjacency) tuples -- onesweep with decoupled look-back.
//
// The reference sorts each thread's m-mer range with nine byte passes, adjacency byte
// first, then the eight k-mer bytes (radixPass, metapart.c:1494-1598, pass order
// :2169-2195), which is a stable sort by (k-mer, adjacency) over the enumeration order.
// Here the whole scan is sorted at once with the same key: lo = kmer << 8 | adj
// (+ hi = kmer >> 56 when 2k + 8 > 64).  One upfront pass histograms every digit; a
// digit whose 256 bins hold all tuples in one bin is skipped (it is constant, e.g. the
// high k-mer bits the m-mer range split fixes).  Each remaining digit is one onesweep
// pass: a CTA ranks its 4096-tuple tile with warp-level multi-split, publishes its digit
// counts, looks back over earlier tiles for its global offsets, reorders the tile in
// shared memory and writes each digit's run contiguously.
#include <dlfcn.h>

#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "k_sort.cuh"

namespace mp {

constexpr int ST = 256;  // threads per tile (three resident tiles per SM)
constexpr int SI = 16;
constexpr int STILE = ST * SI;
constexpr int SW = ST / 32;
constexpr unsigned FULLM = 0xFFFFFFFFu;
constexpr int LB = 4;  // look-back: predecessor status words read per round

struct SortSmem {
    uint64_t keys[STILE];
    uint32_t vals[STILE];
    uint8_t his[STILE];
    uint32_t whist[SW][256];
    uint32_t tstart[256];
    uint64_t gbase[256];
    uint32_t wsum[SW];
    uint32_t tile_id;
    uint32_t nvalid;
    uint32_t seg;         // segment (sample) of the tile
    uint32_t first_tile;  // the segment's first tile: its look-back stops there
    uint64_t base;        // the tile's first tuple
};

__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// One 128-byte-line prefetch per line of [p, p + bytes), spread over a block of `threads`.
__device__ __forceinline__ void prefetch_range(const void *p, uint64_t bytes, int threads)
{
    for (uint64_t off = (uint64_t)threadIdx.x * 128; off < bytes; off += (uint64_t)threads * 128)
        prefetch_l2((const char *)p + off);
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__global__ void __launch_bounds__(256) k_hist_upfront(const uint64_t *__restrict__ lo, const uint8_t *__restrict__ hi,
                                                      uint64_t n, unsigned long long *ghist)
{
    __shared__ uint32_t h[9][256];
    for (int i = threadIdx.x; i < 9 * 256; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t k = lo[i];
#pragma unroll
        for (int b = 0; b < 8; b++) atomicAdd(&h[b][(k >> (8 * b)) & 0xFF], 1u);
        if (hi) atomicAdd(&h[8][hi[i]], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 9 * 256; i += blockDim.x) {
        uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(&ghist[i], (unsigned long long)v);
    }
}

// Digit of a tuple for one pass: SRC 0 = byte of lo at `shift`, 1 = the hi byte,
// 2 = byte of the k-mer value (lo >> 8 | hi << 56) at `shift` (the m-mer bucket digits).
// Opt-in shared memory sizes of the sort kernels, set once per device (thread-safe).
static void sort_kernel_attrs();
static uint32_t onesweep_prefetch_tiles();

template <int SRC>
__device__ __forceinline__ uint32_t digit_of(uint64_t lo, uint32_t hi, int shift)
{
    if (SRC == 0) return (uint32_t)((lo >> shift) & 0xFF);
    if (SRC == 1) return hi;
    return (uint32_t)((((lo >> 8) | ((uint64_t)hi << 56)) >> shift) & 0xFF);
}

// W: ballots per tuple in the ranking, at least the digit's width w (digits are masked to w bits, so
// the planes above w are zero in every lane and filter nothing).
// SEGD: segments (batches of samples) -- the tuple array holds sg.nseg segments one after another, each
// sorted on its own: sg.tstart (nseg + 1 tuple offsets) and sg.tile0 (nseg + 1 tile offsets: a segment's
// tiles start at its first tuple, so no tile spans two segments); a tile's look-back stops at its
// segment's first tile and its digit bases are dbase[seg * sg.dstride + digit].  Without SEGD the array is
// one segment of n tuples (and the kernel keeps its registers for the ranking).
struct Segs {
    const uint32_t *tile0 = nullptr;
    const uint64_t *tstart = nullptr;
    int nseg = 1;
    uint32_t dstride = 0;
};

template <int SRC, int W = 8, bool SEGD = false>
__global__ void __launch_bounds__(ST, 3) k_onesweep(const uint64_t *__restrict__ in_lo, const uint8_t *__restrict__ in_hi,
                                                    const uint32_t *__restrict__ in_id, uint64_t *__restrict__ out_lo,
                                                    uint8_t *__restrict__ out_hi, uint32_t *__restrict__ out_id, uint64_t n,
                                                    int shift, int w, const uint64_t *__restrict__ dbase,
                                                    const uint32_t *__restrict__ nzmask, unsigned long long *status,
                                                    uint32_t *tile_ctr, uint32_t epoch, uint32_t *err, uint32_t pf_tiles,
                                                    unsigned long long *trace, Segs sg, uint32_t spin_cap)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    SortSmem &sm = *reinterpret_cast<SortSmem *>(smraw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t dmask = (1u << w) - 1;
    long long ts[5];  // thread 0's clock at the phase boundaries (trace only; not with segments)
    if constexpr (!SEGD) ts[0] = clock64();
    for (int i = threadIdx.x; i < SW * 256; i += ST) (&sm.whist[0][0])[i] = 0;
    if (threadIdx.x == 0) sm.tile_id = atomicAdd(tile_ctr, 1u);
    __syncthreads();
    if constexpr (SEGD) {  // the segment holding the tile: the last one whose first tile is at or below it
        if (threadIdx.x == 0) {
            const uint32_t t = sm.tile_id;
            int lo = 0, hi = sg.nseg - 1;
            while (lo < hi) {
                const int m = (lo + hi + 1) >> 1;
                if (sg.tile0[m] <= t) lo = m; else hi = m - 1;
            }
            const uint64_t b = sg.tstart[lo] + (uint64_t)(t - sg.tile0[lo]) * STILE;
            sm.seg = (uint32_t)lo;
            sm.first_tile = sg.tile0[lo];
            sm.base = b;
            sm.nvalid = (uint32_t)min((uint64_t)STILE, sg.tstart[lo + 1] - b);
        }
        __syncthreads();
    }
    if constexpr (!SEGD) ts[1] = clock64();
    const uint64_t tile = sm.tile_id;
    const uint64_t base = SEGD ? sm.base : tile * STILE;
    const uint64_t tend = SEGD ? base + sm.nvalid : n;  // the tile's tuples end below tend
    const bool has_hi = in_hi != nullptr;
    if (pf_tiles) {  // the tile that starts pf_tiles later (about one wave of resident tiles) into L2
        const uint64_t pb = base + (uint64_t)pf_tiles * STILE;
        if (pb < n) {
            const uint64_t pn = min((uint64_t)STILE, n - pb);
            prefetch_range(in_lo + pb, pn * 8, ST);
            prefetch_range(in_id + pb, pn * 4, ST);
            if (has_hi) prefetch_range(in_hi + pb, pn, ST);
        }
    }

    uint64_t key[SI];
    uint32_t val[SI], rd[SI];  // rd: rank within the warp's digit (bits 0-15) | digit (bits 16-24, 256 = none)
    uint32_t hv[(SI + 3) / 4];
#pragma unroll
    for (int j = 0; j < (SI + 3) / 4; j++) hv[j] = 0;
#pragma unroll
    for (int j = 0; j < SI; j++) {
        const uint64_t idx = base + (uint64_t)warp * (32 * SI) + (uint64_t)j * 32 + lane;
        const bool v = idx < tend;
        key[j] = v ? in_lo[idx] : 0ull;
        const uint32_t h = (has_hi && v) ? (uint32_t)in_hi[idx] : 0u;
        hv[j >> 2] |= h << (8 * (j & 3));
        rd[j] = (v ? digit_of<SRC>(key[j], h, shift) & dmask : 256u) << 16;
    }
    // warp-level multi-split: stable rank of each tuple among equal digits of its warp.  First every
    // tuple's peers (the lanes holding its digit, from W bit-plane ballots), packed into rd as the
    // peers below its lane (bits 0-4), their number (5-10) and whether it leads them (11); no memory
    // is touched, so the ballots of all tuples issue back to back.  Then one read-modify-write of the
    // warp's running digit count per tuple.
    const uint32_t lt = (1u << lane) - 1;
#pragma unroll
    for (int j = 0; j < SI; j++) {
        const uint32_t d = rd[j] >> 16;
        uint32_t peers = __ballot_sync(FULLM, d < 256);
#pragma unroll
        for (int b = 0; b < W; b++) {
            const uint32_t bb = __ballot_sync(FULLM, (d >> b) & 1u);
            peers &= ((d >> b) & 1u) ? bb : ~bb;
        }
        rd[j] |= (uint32_t)__popc(peers & lt) | ((uint32_t)__popc(peers) << 5) | ((peers & lt) == 0 ? 1u << 11 : 0u);
    }
#pragma unroll
    for (int j = 0; j < SI; j++) {
        const uint32_t d = rd[j] >> 16;
        uint32_t pre = 0;
        if (d < 256) pre = sm.whist[warp][d];
        __syncwarp();
        if (d < 256) {
            if ((rd[j] >> 11) & 1u) sm.whist[warp][d] = pre + ((rd[j] >> 5) & 63u);
            rd[j] = (d << 16) | (pre + (rd[j] & 31u));
        }
        __syncwarp();
    }
    // the ids are needed only for the tile order below: loaded now, they arrive during the digit scan
#pragma unroll
    for (int j = 0; j < SI; j++) {
        // (with segments the tile's bounds are read again: no registers held through the ranking)
        const uint64_t b2 = SEGD ? sm.base : base, e2 = SEGD ? sm.base + sm.nvalid : n;
        const uint64_t idx = b2 + (uint64_t)warp * (32 * SI) + (uint64_t)j * 32 + lane;
        val[j] = idx < e2 ? in_id[idx] : 0u;
    }
    __syncthreads();
    if constexpr (!SEGD) ts[2] = clock64();
    // threads 0..255 own one digit each: warp prefixes, the tile count, its look-back (skipped, with the
    // status word, for a digit that no tuple of the input has: bit clear in nzmask)
    const uint32_t d = threadIdx.x;
    const bool dig = d < 256;
    const bool walk = dig && (!nzmask || ((nzmask[d >> 5] >> (d & 31)) & 1u));
    uint32_t cnt = 0, x = 0;
    if (dig) {
#pragma unroll
        for (int w = 0; w < SW; w++) {
            const uint32_t t = sm.whist[w][d];
            sm.whist[w][d] = cnt;
            cnt += t;
        }
        const unsigned long long E = (unsigned long long)epoch << 60, PF = 1ull << 59;
        const uint64_t first = SEGD ? (uint64_t)sm.first_tile : 0ull;  // the segment's first tile posts a prefix
        if (walk) st_relaxed(status + tile * 256 + d, tile == first ? (E | PF | cnt) : (E | cnt));
        // tile-local exclusive scan of the digit counts (warps 0..7 are all digit owners)
        x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULLM, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sm.wsum[warp] = x;
    }
    __syncthreads();
    if (dig) {
        uint32_t before = 0;
        for (int w = 0; w < warp; w++) before += sm.wsum[w];
        sm.tstart[d] = before + x - cnt;
    }
    if (!SEGD && threadIdx.x == 0) sm.nvalid = (uint32_t)min((uint64_t)STILE, n - base);
    __syncthreads();
    if constexpr (!SEGD) ts[3] = clock64();
    // tile order in shared memory first: the look-back below then finds more predecessors done
#pragma unroll
    for (int j = 0; j < SI; j++) {
        const uint32_t dd = rd[j] >> 16;
        if (dd < 256) {
            const uint32_t s = sm.tstart[dd] + sm.whist[warp][dd] + (rd[j] & 0xFFFF);
            sm.keys[s] = key[j];
            sm.vals[s] = val[j];
            if (has_hi) sm.his[s] = (uint8_t)(hv[j >> 2] >> (8 * (j & 3)));
        }
    }
    uint32_t lb_steps = 0, lb_waits = 0;  // thread 0's look-back: status words summed, polls that found none posted
    if (walk) {
        // decoupled look-back for digit d
        const unsigned long long E = (unsigned long long)epoch << 60, PF = 1ull << 59, CM = PF - 1;
        unsigned long long excl = 0;
        const int64_t first = SEGD ? (int64_t)sm.first_tile : 0;  // before it: prefix 0
        if ((int64_t)tile > first) {
            // LB predecessors' words are read at once, then summed in order up to the first prefix;
            // a word not yet posted ends the round and the next round starts from it
            int64_t p = (int64_t)tile - 1;
            uint32_t spins = 0;
            bool found = false;
            while (!found) {
                unsigned long long v[LB];
#pragma unroll
                for (int q = 0; q < LB; q++) {
                    const int64_t pq = p - q;
                    v[q] = pq >= first ? ld_relaxed(status + (uint64_t)pq * 256 + d) : (E | PF);
                }
                int adv = 0;
                bool stall = false;
#pragma unroll
                for (int q = 0; q < LB; q++) {
                    if (found || stall) continue;
                    if ((v[q] >> 60) != epoch) {
                        stall = true;
                        continue;
                    }
                    excl += v[q] & CM;
                    adv++;
                    found = (v[q] & PF) != 0;
                }
                p -= adv;
                lb_steps += (uint32_t)adv;
                if (stall && !found) {
                    lb_waits++;
                    if (++spins >= spin_cap) {  // spin_cap polls of unposted words at most
                        atomicOr(err, DERR_SPIN);
                        break;
                    }
                }
            }
            st_relaxed(status + tile * 256 + d, E | PF | (excl + cnt));
        }
        sm.gbase[d] = (SEGD ? dbase[(uint64_t)sm.seg * sg.dstride + d] : dbase[d]) + excl;
    }
    __syncthreads();
    if constexpr (!SEGD) ts[4] = clock64();
    const uint32_t nv = sm.nvalid;
    for (uint32_t s = threadIdx.x; s < nv; s += ST) {
        const uint64_t kk = sm.keys[s];
        const uint32_t dd = digit_of<SRC>(kk, has_hi ? sm.his[s] : 0u, shift) & dmask;
        const uint64_t g = sm.gbase[dd] + (s - sm.tstart[dd]);
        if (g >= n) continue;  // only after a failed look-back (err is set)
        out_lo[g] = kk;
        out_id[g] = sm.vals[s];
        if (has_hi) out_hi[g] = sm.his[s];
    }
    // [0] tile id, [1] loads and ranks, [2] digit scan, [3] tile order and look-back, [4] stores (cycles);
    // [5] [6] look-back status words read and polls of unposted words (digit 0)
    if (!SEGD && trace && threadIdx.x == 0) {
        const long long te = clock64();
        for (int q = 0; q < 4; q++) atomicAdd(&trace[q], (unsigned long long)(ts[q + 1] - ts[q]));
        atomicAdd(&trace[4], (unsigned long long)(te - ts[4]));
        atomicAdd(&trace[5], (unsigned long long)lb_steps);
        atomicAdd(&trace[6], (unsigned long long)lb_waits);
    }
}

// Adjacent pairs out of (k-mer, adjacency) order: (hi, lo) compared as one 72-bit key.
__global__ void k_count_unsorted(const uint64_t *lo, const uint8_t *hi, uint64_t n, unsigned long long *out)
{
    unsigned long long c = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ha = hi ? hi[i - 1] : 0u, hb = hi ? hi[i] : 0u;
        c += (ha > hb || (ha == hb && lo[i - 1] > lo[i])) ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(FULLM, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

int count_unsorted(const uint64_t *lo, const uint8_t *hi, uint64_t n, unsigned long long *d_count, cudaStream_t st,
                   uint64_t *out)
{
    MP_CUDA(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    if (n > 1) {
        const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, 8ull * (uint64_t)sm_count());
        (mp::count_launch(), k_count_unsorted<<<(unsigned)blocks, 256, 0, st>>>(lo, hi, n, d_count));
    }
    unsigned long long h = 0;
    MP_CUDA(cudaMemcpyAsync(&h, d_count, sizeof h, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    *out = h;
    return 0;
}

int radix_sort(SortBufs &b, uint64_t n, bool has_hi, DeviceArena &arena, cudaStream_t st, SortStats *stats)
{
    if (stats) *stats = SortStats{};
    if (n <= 1) return 0;
    unsigned long long *ghist = arena.alloc<unsigned long long>(9 * 256);
    uint64_t *dbase = arena.alloc<uint64_t>(9 * 256);
    uint32_t *ctr = arena.alloc<uint32_t>(16);
    uint32_t *err = arena.alloc<uint32_t>(1);
    const uint64_t tiles = (n + STILE - 1) / STILE;
    unsigned long long *status = arena.alloc<unsigned long long>(tiles * 256);
    if (!ghist || !dbase || !ctr || !err || !status) return set_error(MP_ENOMEM, "device memory for the radix sort");
    MP_CUDA(cudaMemsetAsync(ghist, 0, 9 * 256 * sizeof(unsigned long long), st));
    MP_CUDA(cudaMemsetAsync(ctr, 0, 16 * sizeof(uint32_t), st));
    MP_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    MP_CUDA(cudaMemsetAsync(status, 0, tiles * 256 * sizeof(unsigned long long), st));
    Events ht(2);
    cudaEvent_t e0 = ht[0], e1 = ht[1];
    cudaEventRecord(e0, st);
    (mp::count_launch(), k_hist_upfront<<<8 * sm_count(), 256, 0, st>>>(b.lo[b.cur], has_hi ? b.hi[b.cur] : nullptr, n, ghist));
    cudaEventRecord(e1, st);
    std::vector<unsigned long long> h(9 * 256);
    MP_CUDA(cudaMemcpyAsync(h.data(), ghist, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    float hist_ms = 0;
    cudaEventElapsedTime(&hist_ms, e0, e1);
    // digits in LSD order: lo bytes 0..7, then hi
    std::vector<int> passes;
    std::vector<uint64_t> base(9 * 256);
    for (int dgt = 0; dgt < (has_hi ? 9 : 8); dgt++) {
        uint64_t acc = 0;
        bool constant = false;
        for (int v = 0; v < 256; v++) {
            base[dgt * 256 + v] = acc;
            if (h[dgt * 256 + v] == n) constant = true;
            acc += h[dgt * 256 + v];
        }
        if (acc != n) return set_error(MP_EDEVICE, "radix histogram does not add up");
        if (!constant) passes.push_back(dgt);
    }
    MP_CUDA(cudaMemcpyAsync(dbase, base.data(), base.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    sort_kernel_attrs();
    const uint32_t pf = onesweep_prefetch_tiles();
    Events ev(passes.size() + 1);
    cudaEventRecord(ev[0], st);
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const int dgt = passes[pi];
        const int src = b.cur, dst = b.cur ^ 1;
        const uint8_t *ih = has_hi ? b.hi[src] : nullptr;
        uint8_t *oh = has_hi ? b.hi[dst] : nullptr;
        if (dgt < 8)
            (mp::count_launch(), k_onesweep<0><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(b.lo[src], ih, b.id[src], b.lo[dst], oh,
                                                                         b.id[dst], n, 8 * dgt, 8, dbase + dgt * 256, nullptr, status,
                                                                         ctr + pi, (uint32_t)(pi + 1), err, pf, nullptr, Segs{}, arena.lim.lookback_spins));
        else
            (mp::count_launch(), k_onesweep<1><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(b.lo[src], ih, b.id[src], b.lo[dst], oh,
                                                                         b.id[dst], n, 0, 8, dbase + dgt * 256, nullptr, status,
                                                                         ctr + pi, (uint32_t)(pi + 1), err, pf, nullptr, Segs{}, arena.lim.lookback_spins));
        cudaEventRecord(ev[pi + 1], st);
        b.cur = dst;
    }
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (stats) {
        stats->tuples = n;
        stats->passes = (int)passes.size();
        stats->hist_ms = hist_ms;
        for (size_t pi = 0; pi < passes.size(); pi++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[pi], ev[pi + 1]);
            stats->pass_ms += ms;
        }
        const uint64_t elt = 12 + (has_hi ? 1 : 0);
        stats->bytes = (uint64_t)passes.size() * 2 * elt * n;
        stats->hist_bytes = (8 + (has_hi ? 1 : 0)) * n;
    }
    arena.free_scratch(status);
    if (herr) return set_error(MP_EDEVICE, "radix sort look-back gave up (device error flags 0x%x)", herr);
    return 0;
}

// ---------------------------------------------------------------------------
// Sort by m-mer bucket, then within buckets.
//
// The tuples of a scan are sorted first by their m-mer bucket (the top 20 bits of the
// k-mer) with onesweep passes over the bucket bits that vary within the scan, in digits of at
// most 8 bits and near-equal width -- the per-bucket counts are the .kmerHist the scan was
// planned from, so the digit offsets need no histogram pass -- and
// then each unit of consecutive buckets (at most SS_CAP tuples) is sorted in shared memory
// by the rest of the key: (bucket - first bucket of the unit) << lowbits | the low k-mer
// bits and the adjacency byte.  Buckets larger than a unit are gathered, sorted together
// by the device-wide sort and put back.  Both steps are stable, so the result equals the
// stable (k-mer, adjacency) order of the enumeration (metapart.c:1496, 2169-2195).

// Two block shapes sort the units: 512 threads for units of at most SS_SMALL_CAP tuples, two blocks per
// SM (so one block's barriers and digit scans overlap the other's ranking), and 1024 threads, one block
// per SM, for single buckets of up to SS_CAP tuples.  Buckets above SS_CAP take the device-wide sort.
constexpr int SS_ITEMS = 12;
constexpr int SS_CAP = 1024 * SS_ITEMS;        // 12288: the most tuples a unit holds
constexpr int SS_SMALL_CAP = 6128;             // 512 x 12 slots; two blocks' shared memory fit one SM
constexpr uint32_t SS_MAXB = 4096;             // buckets per unit
constexpr int SS_MAXBITS = 9;                  // widest digit of the unit sort (53 varying bits: six passes)
constexpr int SS_BINS = 1 << SS_MAXBITS;

template <int THREADS, int CAP>
struct SegSmemT {
    static constexpr int WARPS = THREADS / 32;
    uint64_t key[CAP];
    uint16_t perm[2][CAP];
    uint32_t ids[CAP];                   // the unit's ids, loaded with the keys
    uint16_t whist[WARPS][SS_BINS];      // digit counts per warp, then each (warp, digit)'s offset in the digit
    uint16_t dstart[SS_BINS];            // first position of each digit
    uint32_t wsum[WARPS];
    unsigned long long kor, kand;
};
typedef SegSmemT<1024, SS_CAP> SegSmemL;
typedef SegSmemT<512, SS_SMALL_CAP> SegSmemS;
static_assert(offsetof(SegSmemL, whist) % 16 == 0 && offsetof(SegSmemS, whist) % 16 == 0,
              "histogram rows are cleared with 16-byte stores");
static_assert(sizeof(SegSmemL) <= 227 * 1024, "one 1024-thread unit block per SM");
static_assert(2 * (sizeof(SegSmemS) + 1024) <= 228 * 1024, "two 512-thread unit blocks per SM");
static_assert(SS_SMALL_CAP <= 512 * SS_ITEMS, "a small unit fits its block's slots");

// One stable counting-sort pass over a unit: perm[cur] (or the identity) -> perm[cur ^ 1] by the
// digit (key >> sh) & mask, nbins = a power of two >= 32 covering the mask.  Items are ranked in
// warp-blocked order with match_any, so equal digits keep their order.  Every warp's histogram row
// is zero on entry and on exit: a warp clears its own row once its scatter has read it.
template <int THREADS, int CAP>
__device__ void seg_pass(SegSmemT<THREADS, CAP> &sm, int cur, uint32_t cnt, int sh, uint32_t mask, uint32_t nbins,
                         bool identity)
{
    constexpr int SS_WARPS = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1;
    uint32_t src[SS_ITEMS], rd[SS_ITEMS];  // rd: rank (bits 0-15) | digit (bits 16-27; nbins = none)
#pragma unroll
    for (int j = 0; j < SS_ITEMS; j++) {
        const uint32_t e = warp * (32 * SS_ITEMS) + j * 32 + lane;
        const bool v = e < cnt;
        src[j] = v ? (identity ? e : (uint32_t)sm.perm[cur][e]) : 0u;
        rd[j] = (v ? (uint32_t)((sm.key[src[j]] >> sh) & mask) : nbins) << 16;
    }
#pragma unroll
    for (int j = 0; j < SS_ITEMS; j++) {
        const uint32_t d = rd[j] >> 16;
        const uint32_t peers = __match_any_sync(FULLM, d);
        uint32_t pre = 0;
        if (d < nbins) pre = sm.whist[warp][d];
        __syncwarp();
        if (d < nbins) {
            rd[j] |= pre + __popc(peers & lt);
            if ((peers & lt) == 0) sm.whist[warp][d] = (uint16_t)(pre + __popc(peers));
        }
        __syncwarp();
    }
    __syncthreads();
    // thread t: digits 2t and 2t + 1 (one 32-bit word of each row): their exclusive prefixes over the warps
    // (into the rows), then their starts
    uint32_t clo = 0, chi = 0, x = 0;
    const uint32_t t = threadIdx.x, npair = nbins / 2;  // nbins >= 32: at least 16 pairs
    if (t < ((npair + 31) & ~31u)) {  // whole warps take part in the shuffles
        if (t < npair) {
#pragma unroll
            for (int w0 = 0; w0 < SS_WARPS; w0 += 8) {
                uint32_t v[8];
#pragma unroll
                for (int i = 0; i < 8; i++) v[i] = reinterpret_cast<const uint32_t *>(sm.whist[w0 + i])[t];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    reinterpret_cast<uint32_t *>(sm.whist[w0 + i])[t] = clo | (chi << 16);
                    clo += v[i] & 0xFFFFu;
                    chi += v[i] >> 16;
                }
            }
        }
        x = clo + chi;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULLM, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sm.wsum[warp] = x;
    }
    __syncthreads();
    if (t < npair) {
        uint32_t before = x - clo - chi;
        for (int w = 0; w < warp; w++) before += sm.wsum[w];
        reinterpret_cast<uint32_t *>(sm.dstart)[t] = before | ((before + clo) << 16);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SS_ITEMS; j++) {
        const uint32_t dd = rd[j] >> 16;
        if (dd < nbins)
            sm.perm[cur ^ 1][(uint32_t)sm.dstart[dd] + sm.whist[warp][dd] + (rd[j] & 0xFFFF)] = (uint16_t)src[j];
    }
    __syncwarp();
    {
        uint4 *row = reinterpret_cast<uint4 *>(&sm.whist[warp][0]);
        for (uint32_t i = lane; i < nbins / 8; i += 32) row[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
}

// Sort of the units, one persistent block per SM: key = (bucket - first bucket of the unit) << lowbits |
// low k-mer bits and adjacency, stable LSD over the key's varying bits in digits of at most max_bits
// (equal widths, so 53 varying bits take six passes).  While a unit is sorted, the next unit of this
// block is prefetched into L2.  trace (nullable): [0] digit passes, [1..3] SM cycles in load, passes, store.
template <int THREADS, int CAP>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) k_segsort(const uint64_t *__restrict__ ustart, const uint32_t *__restrict__ ucount,
                                                         const uint32_t *__restrict__ ubucket, uint32_t nunits,
                                                         const uint64_t *__restrict__ lo_in, const uint8_t *__restrict__ hi_in,
                                                         const uint32_t *__restrict__ id_in, uint64_t *__restrict__ lo_out,
                                                         uint32_t *__restrict__ id_out, int bsh, int lowbits, int max_bits,
                                                         unsigned long long *trace)
{
    constexpr int SS_THREADS = THREADS;
    extern __shared__ __align__(16) unsigned char smraw[];
    SegSmemT<THREADS, CAP> &sm = *reinterpret_cast<SegSmemT<THREADS, CAP> *>(smraw);
    const int lane = threadIdx.x & 31;
    const uint64_t lowmask = (1ull << lowbits) - 1;
    unsigned long long cyc[3] = {0, 0, 0}, npass = 0;
    {
        uint4 *w4 = reinterpret_cast<uint4 *>(&sm.whist[0][0]);
        for (uint32_t i = threadIdx.x; i < sizeof sm.whist / 16; i += SS_THREADS) w4[i] = make_uint4(0, 0, 0, 0);
    }
    for (uint32_t u = blockIdx.x; u < nunits; u += gridDim.x) {
        const long long t0 = clock64();
        const uint64_t start = ustart[u];
        const uint32_t cnt = ucount[u], b0 = ubucket[u] & (NB - 1);  // the first bucket within its segment
        if (u + gridDim.x < nunits) {
            const uint64_t ns = ustart[u + gridDim.x], nc = ucount[u + gridDim.x];
            prefetch_range(lo_in + ns, nc * 8, SS_THREADS);
            prefetch_range(id_in + ns, nc * 4, SS_THREADS);
            if (hi_in) prefetch_range(hi_in + ns, nc, SS_THREADS);
        }
        if (threadIdx.x == 0) {
            sm.kor = 0;
            sm.kand = ~0ull;
        }
        // all loads of the unit in flight at once
        uint64_t lr[SS_ITEMS];
        uint32_t hr[SS_ITEMS], ir[SS_ITEMS];
#pragma unroll
        for (int j = 0; j < SS_ITEMS; j++) {
            const uint32_t e = threadIdx.x + j * SS_THREADS;
            lr[j] = e < cnt ? lo_in[start + e] : 0ull;
            hr[j] = (hi_in && e < cnt) ? (uint32_t)hi_in[start + e] : 0u;
            ir[j] = e < cnt ? id_in[start + e] : 0u;
        }
        __syncthreads();
        unsigned long long kor = 0, kand = ~0ull;
#pragma unroll
        for (int j = 0; j < SS_ITEMS; j++) {
            const uint32_t e = threadIdx.x + j * SS_THREADS;
            if (e < cnt) {
                const uint64_t km = (lr[j] >> 8) | ((uint64_t)hr[j] << 56);
                const uint64_t key = ((uint64_t)((uint32_t)(km >> bsh) - b0) << lowbits) | (lr[j] & lowmask);
                sm.key[e] = key;
                sm.ids[e] = ir[j];
                kor |= key;
                kand &= key;
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            kor |= __shfl_xor_sync(FULLM, kor, o);
            kand &= __shfl_xor_sync(FULLM, kand, o);
        }
        if (lane == 0) {
            atomicOr(&sm.kor, kor);
            atomicAnd(&sm.kand, kand);
        }
        __syncthreads();
        const long long t1 = clock64();
        const uint64_t varying = sm.kor ^ sm.kand;
        int cur = -1;  // -1: the identity order
        if (varying) {
            const int lb = __ffsll((long long)varying) - 1, hb = 63 - __clzll((long long)varying);
            const int span = hb - lb + 1, np = (span + max_bits - 1) / max_bits, w = (span + np - 1) / np;
            const uint32_t mask = (uint32_t)((1ull << w) - 1), nbins = (1u << w) < 32u ? 32u : (1u << w);
            int c = 0;
            for (int i = 0; i < np; i++) {
                const int sh = lb + i * w;
                if (!((varying >> sh) & mask)) continue;  // constant digit in this unit
                seg_pass(sm, c, cnt, sh, mask, nbins, cur < 0);
                c ^= 1;
                cur = c;
                npass++;
            }
        }
        const long long t2 = clock64();
        for (uint32_t e = threadIdx.x; e < cnt; e += SS_THREADS) {
            const uint32_t sidx = cur < 0 ? e : (uint32_t)sm.perm[cur][e];
            const uint64_t key = sm.key[sidx];
            const uint64_t bucket = b0 + (key >> lowbits);
            lo_out[start + e] = (bucket << lowbits) | (key & lowmask);
            id_out[start + e] = sm.ids[sidx];
        }
        __syncthreads();  // the next unit reuses the shared arrays
        cyc[0] += (unsigned long long)(t1 - t0);
        cyc[1] += (unsigned long long)(t2 - t1);
        cyc[2] += (unsigned long long)(clock64() - t2);
    }
    if (trace && threadIdx.x == 0) {
        atomicAdd(&trace[0], npass);
        for (int q = 0; q < 3; q++) atomicAdd(&trace[1 + q], cyc[q]);
    }
}

// Big buckets: gather with key (big-bucket index << lowbits | low bits), sort, put back.
__global__ void k_big_gather(const uint64_t *__restrict__ bstart, const uint32_t *__restrict__ bcount,
                             const uint64_t *__restrict__ boff, const uint64_t *__restrict__ lo_in,
                             const uint32_t *__restrict__ id_in, uint64_t *__restrict__ tk, uint32_t *__restrict__ tid,
                             int lowbits)
{
    const uint32_t b = blockIdx.x;
    const uint64_t lowmask = (1ull << lowbits) - 1, s = bstart[b], o = boff[b];
    for (uint32_t e = threadIdx.x; e < bcount[b]; e += blockDim.x) {
        tk[o + e] = ((uint64_t)b << lowbits) | (lo_in[s + e] & lowmask);
        tid[o + e] = id_in[s + e];
    }
}

__global__ void k_big_scatter(const uint64_t *__restrict__ bstart, const uint32_t *__restrict__ bcount,
                              const uint32_t *__restrict__ bbucket, const uint64_t *__restrict__ boff,
                              const uint64_t *__restrict__ tk, const uint32_t *__restrict__ tid, uint64_t *__restrict__ lo_out,
                              uint32_t *__restrict__ id_out, int lowbits)
{
    const uint32_t b = blockIdx.x;
    const uint64_t lowmask = (1ull << lowbits) - 1, s = bstart[b], o = boff[b];
    const uint64_t hibits = (uint64_t)(bbucket[b] & (NB - 1)) << lowbits;  // the bucket within its segment
    for (uint32_t e = threadIdx.x; e < bcount[b]; e += blockDim.x) {
        lo_out[s + e] = hibits | (tk[o + e] & lowmask);
        id_out[s + e] = tid[o + e];
    }
}

// ---- planning of one scan's bucket sort on the device, from the .kmerHist prefix (d_hist, 1048577 u64)


// The bucket-digit passes of one scan: pass p sorts by the bucket bits [sh[p], sh[p] + w[p]), w <= 8.
struct BucketPasses {
    int np;
    int sh[3], w[3];
};

// Digit counts of the passes (weighted by the bucket counts) and the populated-bucket flags.  A block takes
// BP_CHUNK consecutive buckets from lo; with segments (lo = 0) the chunk lies in one segment's NB buckets,
// whose counts go to that segment's rows: dcnt[(seg * 3 + pass) * 256 + digit].
constexpr uint64_t BP_CHUNK = 4096;
static_assert(NB % BP_CHUNK == 0, "a chunk of buckets never spans two segments");

__global__ void __launch_bounds__(256) k_bp_count(const uint64_t *__restrict__ hist, uint64_t lo, uint64_t nbk,
                                                  BucketPasses bp, bool segmented, unsigned long long *dcnt,
                                                  uint32_t *pop)
{
    __shared__ unsigned long long h[3 * 256];
    for (int i = threadIdx.x; i < 3 * 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint64_t c0 = (uint64_t)blockIdx.x * BP_CHUNK, c1 = min(nbk, c0 + BP_CHUNK);
    const uint64_t seg = segmented ? ((lo + c0) / NB) : 0;
    for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
        const uint64_t b = lo + i, c = hist[b + 1] - hist[b];
        pop[i] = c ? 1u : 0u;
        if (!c) continue;
        const uint32_t lb = (uint32_t)(b & (NB - 1));  // the bucket within its segment
#pragma unroll
        for (int p = 0; p < 3; p++)
            if (p < bp.np) atomicAdd(&h[p * 256 + ((lb >> bp.sh[p]) & ((1u << bp.w[p]) - 1))], (unsigned long long)c);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < bp.np * 256; i += blockDim.x)
        if (h[i]) atomicAdd(&dcnt[seg * 3 * 256 + i], h[i]);
}

// Per (segment, pass), one block of 256: digit offsets (the segment's first tuple plus the exclusive digit
// prefix), the digits that occur (ORed over the segments), the largest digit count and the total.
__global__ void __launch_bounds__(256) k_bp_digits(const unsigned long long *dcnt, int np, const uint64_t *tstart,
                                                   uint64_t *dbase, uint32_t *dnz, unsigned long long *dmax,
                                                   unsigned long long *dtot)
{
    __shared__ unsigned long long ws[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int seg = blockIdx.x / np, p = blockIdx.x % np;
    const uint64_t row = (uint64_t)seg * 3 + p;
    const unsigned long long c = dcnt[row * 256 + threadIdx.x];
    unsigned long long x = c, m = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(FULLM, x, o);
        if (lane >= o) x += y;
        m = max(m, __shfl_xor_sync(FULLM, m, o));
    }
    const uint32_t nzw = __ballot_sync(FULLM, c != 0);
    if (lane == 0 && nzw) atomicOr(&dnz[p * 8 + warp], nzw);
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    unsigned long long before = 0;
    for (int q = 0; q < warp; q++) before += ws[q];
    dbase[row * 256 + threadIdx.x] = (tstart ? tstart[seg] : 0ull) + before + x - c;
    if (threadIdx.x == 255) dtot[row] = before + x;
    __syncthreads();
    if (lane == 0) ws[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long mm = 0;
        for (int q = 0; q < 8; q++) mm = max(mm, ws[q]);
        dmax[row] = mm;
    }
}

__global__ void k_bp_compact(const uint32_t *pop, const uint64_t *popoff, uint64_t lo, uint64_t nbk, uint32_t *P)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nbk && pop[i]) P[popoff[i]] = (uint32_t)(lo + i);
}

constexpr int BP_BLOCK = 256;  // populated buckets packed greedily by one thread

// Greedy packing of consecutive populated buckets into units (at most cap tuples, SS_MAXB buckets, all
// of one segment), one thread per block of BP_BLOCK populated buckets; buckets above cap are listed
// apart.  Units never cross a block, so each block ends with one partial unit.  Block g writes its units from g * BP_BLOCK
// into the staging arrays and their counts to nu_blk[g], nb_blk[g].
__global__ void k_bp_greedy(const uint32_t *P, uint64_t np, const uint64_t *__restrict__ hist, uint64_t lo,
                            uint64_t *sus, uint32_t *suc, uint32_t *sub, uint64_t *sbs, uint32_t *sbc, uint32_t *sbb,
                            uint32_t *nu_blk, uint32_t *nb_blk, uint32_t cap)
{
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t i0 = g * BP_BLOCK;
    if (i0 >= np) return;
    const uint64_t i1 = min(np, i0 + BP_BLOCK), base = hist[lo];
    uint32_t nu = 0, nb = 0, u_b0 = 0;
    uint64_t u_start = 0, u_cnt = 0;
    bool have = false;
    for (uint64_t i = i0; i < i1; i++) {
        const uint64_t bk = P[i], c = hist[bk + 1] - hist[bk], s = hist[bk] - base;
        if (c > (uint64_t)cap) {
            if (have) {
                sus[i0 + nu] = u_start; suc[i0 + nu] = (uint32_t)u_cnt; sub[i0 + nu] = u_b0; nu++;
                have = false;
            }
            sbs[i0 + nb] = s; sbc[i0 + nb] = (uint32_t)c; sbb[i0 + nb] = (uint32_t)bk; nb++;
            continue;
        }
        if (have && (u_cnt + c > (uint64_t)cap || bk - u_b0 >= SS_MAXB || bk / NB != u_b0 / NB)) {
            sus[i0 + nu] = u_start; suc[i0 + nu] = (uint32_t)u_cnt; sub[i0 + nu] = u_b0; nu++;
            have = false;
        }
        if (!have) {
            have = true;
            u_start = s;
            u_cnt = 0;
            u_b0 = (uint32_t)bk;
        }
        u_cnt += c;
    }
    if (have) { sus[i0 + nu] = u_start; suc[i0 + nu] = (uint32_t)u_cnt; sub[i0 + nu] = u_b0; nu++; }
    nu_blk[g] = nu;
    nb_blk[g] = nb;
}

// Staged per-block units and oversized buckets into dense arrays (offsets from scans of the block counts).
__global__ void k_bp_gather(uint64_t nblk, const uint32_t *nu_blk, const uint64_t *uoff, const uint32_t *nb_blk,
                            const uint64_t *boff, const uint64_t *sus, const uint32_t *suc, const uint32_t *sub,
                            const uint64_t *sbs, const uint32_t *sbc, const uint32_t *sbb, uint64_t *us, uint32_t *uc,
                            uint32_t *ub, uint64_t *bs, uint32_t *bc, uint32_t *bb)
{
    const uint64_t g = blockIdx.x;
    if (g >= nblk) return;
    const uint64_t i0 = g * BP_BLOCK;
    for (uint32_t q = threadIdx.x; q < nu_blk[g]; q += blockDim.x) {
        us[uoff[g] + q] = sus[i0 + q];
        uc[uoff[g] + q] = suc[i0 + q];
        ub[uoff[g] + q] = sub[i0 + q];
    }
    for (uint32_t q = threadIdx.x; q < nb_blk[g]; q += blockDim.x) {
        bs[boff[g] + q] = sbs[i0 + q];
        bc[boff[g] + q] = sbc[i0 + q];
        bb[boff[g] + q] = sbb[i0 + q];
    }
}

// ---- the bucket sort's plan knobs, by k and scan size
//
// Three knobs shape the bucket sort: the bucket digits (the scan's varying bits in passes of near-equal
// width, or the bucket's bytes: MP_SORT_BUCKET_DIGITS=bytes), the unit sort's widest digit (5..9 bits:
// MP_UNIT_SORT_MAX_BITS) and how far ahead a digit-pass tile prefetches its successor (SM waves:
// MP_ONESWEEP_PF_WAVES, 0 = none).  Their values come from the environment when set, else from the table
// the autotuner (metapart_gb300/autotune.py) measured -- rows "k min_tuples digits unit_bits pf_waves",
// the row of the nearest k and the largest min_tuples not above the scan's tuples -- read once per process
// from MP_SORT_TUNING or sort_tuning.tsv one directory above the library, else the defaults below (one
// wave ahead measured best at 20M reads: 57.8 ms for the digit passes at one wave, 58.4 at two, 60.6 at
// three, 64.6 without).
struct SortTuning {
    bool byte_digits = false;
    int unit_bits = SS_MAXBITS;
    int pf_waves = 1;
};

struct TuneRow {
    int k;
    uint64_t min_tuples;
    SortTuning t;
};

static std::vector<TuneRow> g_tune;
static std::once_flag g_tune_once;

static void load_tuning()
{
    std::string path;
    const char *e = getenv("MP_SORT_TUNING");
    if (e && *e) {
        path = e;
    } else {
        Dl_info info;
        if (dladdr((void *)&load_tuning, &info) && info.dli_fname) {
            path = info.dli_fname;
            const size_t cut = path.find_last_of('/');
            path = (cut == std::string::npos ? std::string(".") : path.substr(0, cut)) + "/../sort_tuning.tsv";
        }
    }
    FILE *f = path.empty() ? nullptr : fopen(path.c_str(), "r");
    if (!f) return;
    char line[256];
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '#') continue;
        int k = 0, bits = 0, pf = 0;
        unsigned long long mt = 0;
        char dig[32] = {0};
        if (sscanf(line, "%d %llu %31s %d %d", &k, &mt, dig, &bits, &pf) != 5) continue;
        TuneRow r;
        r.k = k;
        r.min_tuples = mt;
        r.t.byte_digits = std::string(dig) == "bytes";
        r.t.unit_bits = bits < 5 ? 5 : (bits > SS_MAXBITS ? SS_MAXBITS : bits);
        r.t.pf_waves = pf < 0 ? 0 : (pf > 16 ? 16 : pf);
        g_tune.push_back(r);
    }
    fclose(f);
}

static SortTuning sort_tuning(int k, uint64_t n)
{
    std::call_once(g_tune_once, load_tuning);
    SortTuning t;
    int bk = -1;
    uint64_t bmt = 0;
    for (const TuneRow &r : g_tune) {  // nearest k, then the largest min_tuples <= n
        const int dk = std::abs(r.k - k), dbk = bk < 0 ? 1 << 30 : std::abs(bk - k);
        if (r.min_tuples > n || dk > dbk) continue;
        if (dk < dbk || r.min_tuples >= bmt) {
            t = r.t;
            bk = r.k;
            bmt = r.min_tuples;
        }
    }
    const char *e = getenv("MP_SORT_BUCKET_DIGITS");
    if (e && *e) t.byte_digits = std::string(e) == "bytes";
    e = getenv("MP_UNIT_SORT_MAX_BITS");
    if (e && *e) {
        const int v = atoi(e);
        t.unit_bits = v < 5 ? 5 : (v > SS_MAXBITS ? SS_MAXBITS : v);
    }
    e = getenv("MP_ONESWEEP_PF_WAVES");
    if (e && *e) {
        const int w = atoi(e);
        t.pf_waves = w < 0 ? 0 : (w > 16 ? 16 : w);
    }
    return t;
}

// Prefetch distance of the device-wide sort (no k or scan plan): MP_ONESWEEP_PF_WAVES or one wave.
static uint32_t onesweep_prefetch_tiles()
{
    const char *e = getenv("MP_ONESWEEP_PF_WAVES");
    int w = e && *e ? atoi(e) : 1;
    w = w < 0 ? 0 : (w > 16 ? 16 : w);
    return (uint32_t)w * (uint32_t)sm_count();
}

static void sort_kernel_attrs()
{
    static std::once_flag once[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::call_once(once[dev & 63], [] {
        cudaFuncSetAttribute(k_onesweep<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 7, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 6, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<2, 5, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_segsort<1024, SS_CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SegSmemL));
        cudaFuncSetAttribute(k_segsort<512, SS_SMALL_CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SegSmemS));
    });
}

int bucket_sort(SortBufs &b, uint64_t n, bool has_hi, int k, const uint64_t *d_hist, uint64_t scan_lo, uint64_t scan_hi,
                DeviceArena &arena, cudaStream_t st, SortStats *stats, int *out_lo_buf, int *out_hi_buf,
                const SortSegments *segs)
{
    if (stats) *stats = SortStats{};
    *out_lo_buf = *out_hi_buf = b.cur;
    if (n <= 1) return 0;
    if (scan_hi <= scan_lo) return set_error(MP_EFMT, "the histogram does not match the scan's tuples");
    const int nseg = segs ? segs->nseg : 1;
    if (segs && (scan_lo != 0 || scan_hi != (uint64_t)nseg * NB || (int)segs->tstart.size() != nseg + 1))
        return set_error(MP_EARG, "segmented bucket sort: the buckets must be the segments' NB each");
    const int bsh = 2 * (k - 10), lowbits = 2 * (k - 10) + 8;
    const uint64_t nbk = scan_hi - scan_lo;
    const SortTuning tune = sort_tuning(k, n);
    // ---- plan on the device: digit offsets of the passes, populated buckets.  The scan's varying bucket
    // bits (those of scan_lo ^ (scan_hi - 1); every bucket bit with segments) are split into the fewest
    // passes of at most 8 bits, of near-equal widths (19 bits: 7 + 6 + 6), so no pass ranks or looks back
    // over digits that cannot occur; MP_SORT_BUCKET_DIGITS=bytes takes the bucket's bytes instead.
    BucketPasses bpl{};
    {
        int vb = 0;
        for (uint64_t v = segs ? (uint64_t)(NB - 1) : (scan_lo ^ (scan_hi - 1)); v; v >>= 1) vb++;
        if (tune.byte_digits) {
            bpl.np = 3;
            for (int p = 0; p < 3; p++) bpl.sh[p] = 8 * p, bpl.w[p] = 8;
        } else {
            bpl.np = vb ? (vb + 7) / 8 : 1;
            const int wb = vb / bpl.np, extra = vb % bpl.np;
            for (int p = 0, at = 0; p < bpl.np; p++) {
                bpl.w[p] = wb + (p < extra ? 1 : 0);
                if (bpl.w[p] < 1) bpl.w[p] = 1;
                bpl.sh[p] = at;
                at += bpl.w[p];
            }
        }
    }
    const uint64_t rows = (uint64_t)nseg * 3;
    unsigned long long *dcnt = arena.alloc<unsigned long long>(rows * 256), *dmax = arena.alloc<unsigned long long>(2 * rows);
    uint64_t *dbase = arena.alloc<uint64_t>(rows * 256), *tot = arena.alloc<uint64_t>(4), *popoff = arena.alloc<uint64_t>(nbk + 2);
    uint32_t *dnz = arena.alloc<uint32_t>(3 * 8), *pop = arena.alloc<uint32_t>(nbk + 1);
    const size_t tbp = scan_tmp_bytes(nbk + 1);
    void *tmp = arena.alloc<uint8_t>(tbp);
    uint64_t *d_tstart = segs ? arena.alloc<uint64_t>(nseg + 1) : nullptr;
    uint32_t *d_tile0 = segs ? arena.alloc<uint32_t>(nseg + 1) : nullptr;
    if (!dcnt || !dmax || !dbase || !tot || !popoff || !dnz || !pop || !tmp || (segs && (!d_tstart || !d_tile0)))
        return set_error(MP_ENOMEM, "device memory for the bucket sort");
    // tiles: each segment's own, from its first tuple
    uint64_t tiles = (n + STILE - 1) / STILE;
    if (segs) {
        std::vector<uint32_t> t0(nseg + 1, 0);
        uint64_t acc = 0;
        for (int q = 0; q < nseg; q++) {
            t0[q] = (uint32_t)acc;
            acc += (segs->tstart[q + 1] - segs->tstart[q] + STILE - 1) / STILE;
        }
        t0[nseg] = (uint32_t)acc;
        if (acc >= 0xFFFFFFFFull || segs->tstart[nseg] != n) return set_error(MP_EARG, "segmented bucket sort: bad segments");
        tiles = acc;
        MP_CUDA(cudaMemcpyAsync(d_tstart, segs->tstart.data(), (nseg + 1) * 8, cudaMemcpyHostToDevice, st));
        MP_CUDA(cudaMemcpyAsync(d_tile0, t0.data(), (nseg + 1) * 4, cudaMemcpyHostToDevice, st));
    }
    MP_CUDA(cudaMemsetAsync(dcnt, 0, rows * 256 * sizeof(unsigned long long), st));
    MP_CUDA(cudaMemsetAsync(dnz, 0, 3 * 8 * sizeof(uint32_t), st));
    MP_CUDA(cudaMemsetAsync(pop + nbk, 0, sizeof(uint32_t), st));
    (mp::count_launch(), k_bp_count<<<(unsigned)((nbk + BP_CHUNK - 1) / BP_CHUNK), 256, 0, st>>>(d_hist, scan_lo, nbk, bpl,
                                                                                              segs != nullptr, dcnt, pop));
    (mp::count_launch(), k_bp_digits<<<(unsigned)(nseg * bpl.np), 256, 0, st>>>(dcnt, bpl.np, d_tstart, dbase, dnz, dmax,
                                                                             dmax + rows));
    scan_u32_to_u64(pop, popoff, nbk + 1, tot, tmp, tbp, st);
    uint64_t hd = 0;  // populated buckets
    std::vector<unsigned long long> hm(2 * rows);  // per (segment, pass): largest digit count, then the totals
    MP_CUDA(cudaMemcpyAsync(&hd, tot, 8, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaMemcpyAsync(hm.data(), dmax, hm.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    {
        uint64_t total = 0;
        for (int q = 0; q < nseg; q++) {
            const unsigned long long t = hm[rows + (uint64_t)q * 3];
            if (segs && t != segs->tstart[q + 1] - segs->tstart[q])
                return set_error(MP_EFMT, "the histogram does not match segment %d's tuples", q);
            total += t;
        }
        if (total != n) return set_error(MP_EFMT, "the histogram does not match the scan's tuples");
    }
    const uint64_t np = hd;
    std::vector<int> passes;  // a pass runs unless its digit is constant within every segment
    for (int d = 0; d < bpl.np; d++) {
        bool constant = true;
        for (int q = 0; q < nseg && constant; q++)
            constant = hm[(uint64_t)q * 3 + d] == hm[rows + (uint64_t)q * 3 + d];
        if (!constant) passes.push_back(d);
    }
    uint32_t *ctr = arena.alloc<uint32_t>(8), *err = arena.alloc<uint32_t>(1);
    unsigned long long *trace = arena.alloc<unsigned long long>(16);  // [0..3] unit sort, [8..12] digit passes
    unsigned long long *status = passes.empty() ? nullptr : arena.alloc<unsigned long long>(tiles * 256);
    if (!ctr || !err || !trace || (!passes.empty() && !status)) return set_error(MP_ENOMEM, "device memory for the bucket sort");
    MP_CUDA(cudaMemsetAsync(trace, 0, 16 * sizeof(unsigned long long), st));
    MP_CUDA(cudaMemsetAsync(ctr, 0, 8 * sizeof(uint32_t), st));
    MP_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    if (status) MP_CUDA(cudaMemsetAsync(status, 0, tiles * 256 * sizeof(unsigned long long), st));
    sort_kernel_attrs();
    const uint32_t pf = (uint32_t)tune.pf_waves * (uint32_t)sm_count();
    Segs sg;
    if (segs) {
        sg.tile0 = d_tile0;
        sg.tstart = d_tstart;
        sg.nseg = nseg;
        sg.dstride = 3 * 256;
    }
    Events ev(5);
    cudaEventRecord(ev[0], st);
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const int d = passes[pi];
        const int src = b.cur, dst = b.cur ^ 1;
        const int w = bpl.w[d];
        auto kern = segs ? (w >= 8 ? k_onesweep<2, 8, true> : w == 7 ? k_onesweep<2, 7, true> : w == 6 ? k_onesweep<2, 6, true>
                                                                                               : k_onesweep<2, 5, true>)
                         : (w >= 8 ? k_onesweep<2, 8> : w == 7 ? k_onesweep<2, 7> : w == 6 ? k_onesweep<2, 6> : k_onesweep<2, 5>);
        (mp::count_launch(), kern<<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(
            b.lo[src], has_hi ? b.hi[src] : nullptr, b.id[src], b.lo[dst], has_hi ? b.hi[dst] : nullptr, b.id[dst], n,
            bsh + bpl.sh[d], bpl.w[d], dbase + d * 256, dnz + d * 8, status, ctr + pi, (uint32_t)(pi + 1), err, pf,
            trace + 8, sg, arena.lim.lookback_spins));
        b.cur = dst;
    }
    cudaEventRecord(ev[1], st);
    // ---- units of consecutive buckets and the oversized buckets, planned on the device
    const uint64_t nblk = (np + BP_BLOCK - 1) / BP_BLOCK;
    const uint64_t cap = nblk * BP_BLOCK + 1;
    uint32_t *P = arena.alloc<uint32_t>(np + 1), *nu_blk = arena.alloc<uint32_t>(nblk + 1), *nb_blk = arena.alloc<uint32_t>(nblk + 1);
    uint64_t *uoff = arena.alloc<uint64_t>(nblk + 2), *boff = arena.alloc<uint64_t>(nblk + 2);
    uint64_t *s_us = arena.alloc<uint64_t>(cap), *s_bs = arena.alloc<uint64_t>(cap);
    uint32_t *s_uc = arena.alloc<uint32_t>(cap), *s_ub = arena.alloc<uint32_t>(cap);
    uint32_t *s_bc = arena.alloc<uint32_t>(cap), *s_bb = arena.alloc<uint32_t>(cap);
    uint64_t *d_us = arena.alloc<uint64_t>(np + 1), *d_bs = arena.alloc<uint64_t>(np + 1);
    uint32_t *d_uc = arena.alloc<uint32_t>(np + 1), *d_ub = arena.alloc<uint32_t>(np + 1);
    uint32_t *d_bc = arena.alloc<uint32_t>(np + 1), *d_bb = arena.alloc<uint32_t>(np + 1);
    const size_t tb2 = scan_tmp_bytes(nblk + 1);
    void *tmp2 = arena.alloc<uint8_t>(tb2), *tmp3 = arena.alloc<uint8_t>(tb2);
    if (!P || !nu_blk || !nb_blk || !uoff || !boff || !s_us || !s_bs || !s_uc || !s_ub || !s_bc || !s_bb || !d_us || !d_bs ||
        !d_uc || !d_ub || !d_bc || !d_bb || !tmp2 || !tmp3)
        return set_error(MP_ENOMEM, "device memory for sort units");
    (mp::count_launch(), k_bp_compact<<<(unsigned)((nbk + 255) / 256), 256, 0, st>>>(pop, popoff, scan_lo, nbk, P));
    MP_CUDA(cudaMemsetAsync(nu_blk, 0, (nblk + 1) * sizeof(uint32_t), st));
    MP_CUDA(cudaMemsetAsync(nb_blk, 0, (nblk + 1) * sizeof(uint32_t), st));
    if (nblk) {
        (mp::count_launch(), k_bp_greedy<<<(unsigned)((nblk + 127) / 128), 128, 0, st>>>(P, np, d_hist, scan_lo, s_us, s_uc, s_ub,
                                                                                      s_bs, s_bc, s_bb, nu_blk, nb_blk,
                                                                                      (uint32_t)SS_SMALL_CAP));
    }
    scan_u32_to_u64(nu_blk, uoff, nblk + 1, tot + 1, tmp2, tb2, st);
    scan_u32_to_u64(nb_blk, boff, nblk + 1, tot + 2, tmp3, tb2, st);
    if (nblk)
        (mp::count_launch(), k_bp_gather<<<(unsigned)nblk, 128, 0, st>>>(nblk, nu_blk, uoff, nb_blk, boff, s_us, s_uc, s_ub, s_bs,
                                                                       s_bc, s_bb, d_us, d_uc, d_ub, d_bs, d_bc, d_bb));
    uint64_t hn[2] = {0, 0};
    MP_CUDA(cudaMemcpyAsync(hn, tot + 1, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    const uint64_t nu = hn[0];
    uint64_t nb = hn[1], nm = 0;
    const int in = b.cur, out = b.cur ^ 1;
    if (nu)
        (mp::count_launch(), k_segsort<512, SS_SMALL_CAP><<<(unsigned)std::min<uint64_t>(nu, 2ull * (uint64_t)sm_count()), 512,
                                                            sizeof(SegSmemS), st>>>(
            d_us, d_uc, d_ub, (uint32_t)nu, b.lo[in], has_hi ? b.hi[in] : nullptr, b.id[in], b.lo[out], b.id[out], bsh,
            lowbits, tune.unit_bits, trace));
    // buckets above a small unit: up to SS_CAP tuples each is a unit of its own for the 1024-thread blocks,
    // the rest take the device-wide sort
    std::vector<uint32_t> bc;
    if (nb) {
        std::vector<uint64_t> hs(nb);
        std::vector<uint32_t> hc(nb), hk(nb);
        MP_CUDA(cudaMemcpyAsync(hs.data(), d_bs, nb * 8, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(hc.data(), d_bc, nb * 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(hk.data(), d_bb, nb * 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        std::vector<uint64_t> ms, gs;
        std::vector<uint32_t> mc, mk, gk;
        for (uint64_t q = 0; q < nb; q++) {
            if (hc[q] <= (uint32_t)SS_CAP) {
                ms.push_back(hs[q]);
                mc.push_back(hc[q]);
                mk.push_back(hk[q]);
            } else {
                gs.push_back(hs[q]);
                bc.push_back(hc[q]);
                gk.push_back(hk[q]);
            }
        }
        nm = ms.size();
        nb = gs.size();
        if (nm) {
            uint64_t *d_ms = arena.alloc<uint64_t>(nm);
            uint32_t *d_mc = arena.alloc<uint32_t>(nm), *d_mk = arena.alloc<uint32_t>(nm);
            if (!d_ms || !d_mc || !d_mk) return set_error(MP_ENOMEM, "device memory for sort units");
            MP_CUDA(cudaMemcpyAsync(d_ms, ms.data(), nm * 8, cudaMemcpyHostToDevice, st));
            MP_CUDA(cudaMemcpyAsync(d_mc, mc.data(), nm * 4, cudaMemcpyHostToDevice, st));
            MP_CUDA(cudaMemcpyAsync(d_mk, mk.data(), nm * 4, cudaMemcpyHostToDevice, st));
            (mp::count_launch(), k_segsort<1024, SS_CAP><<<(unsigned)std::min<uint64_t>(nm, (uint64_t)sm_count()), 1024,
                                                          sizeof(SegSmemL), st>>>(
                d_ms, d_mc, d_mk, (uint32_t)nm, b.lo[in], has_hi ? b.hi[in] : nullptr, b.id[in], b.lo[out], b.id[out], bsh,
                lowbits, tune.unit_bits, trace));
        }
        if (nb) {  // the oversized buckets, in order, at the front of the lists
            MP_CUDA(cudaMemcpyAsync(d_bs, gs.data(), nb * 8, cudaMemcpyHostToDevice, st));
            MP_CUDA(cudaMemcpyAsync(d_bc, bc.data(), nb * 4, cudaMemcpyHostToDevice, st));
            MP_CUDA(cudaMemcpyAsync(d_bb, gk.data(), nb * 4, cudaMemcpyHostToDevice, st));
            MP_CUDA(cudaStreamSynchronize(st));  // gs, bc and gk are host vectors of this block
        }
    }
    cudaEventRecord(ev[2], st);
    uint64_t nbig = 0;
    if (nb) {
        std::vector<uint64_t> bo(nb);
        uint64_t *d_bo = arena.alloc<uint64_t>(nb + 1);
        if (!d_bo) return set_error(MP_ENOMEM, "device memory for oversized buckets");
        // batches of oversized buckets whose index fits above the low key bits
        const size_t per_batch = lowbits >= 44 ? ((size_t)1 << (64 - lowbits)) : ((size_t)1 << 20);
        uint64_t maxbatch = 0;
        for (size_t b0 = 0; b0 < nb; b0 += per_batch) {
            uint64_t t = 0;
            for (size_t q = b0; q < nb && q < b0 + per_batch; q++) t += bc[q];
            if (t > maxbatch) maxbatch = t;
            nbig += t;
        }
        SortBufs t;
        for (int q = 0; q < 2; q++) {
            t.lo[q] = arena.alloc<uint64_t>(maxbatch + 1);
            t.id[q] = arena.alloc<uint32_t>(maxbatch + 1);
            if (!t.lo[q] || !t.id[q]) return set_error(MP_ENOMEM, "device memory for oversized buckets");
        }
        for (size_t b0 = 0; b0 < nb; b0 += per_batch) {
            const size_t b1 = std::min<size_t>(nb, b0 + per_batch);
            uint64_t acc = 0;
            for (size_t q = b0; q < b1; q++) { bo[q] = acc; acc += bc[q]; }
            MP_CUDA(cudaMemcpyAsync(d_bo + b0, bo.data() + b0, (b1 - b0) * 8, cudaMemcpyHostToDevice, st));
            t.cur = 0;
            (mp::count_launch(), k_big_gather<<<(unsigned)(b1 - b0), 256, 0, st>>>(d_bs + b0, d_bc + b0, d_bo + b0, b.lo[in],
                                                                                  b.id[in], t.lo[0], t.id[0], lowbits));
            SortStats bst;
            int rc = radix_sort(t, acc, false, arena, st, &bst);
            if (rc) return rc;
            (mp::count_launch(), k_big_scatter<<<(unsigned)(b1 - b0), 256, 0, st>>>(d_bs + b0, d_bc + b0, d_bb + b0, d_bo + b0,
                                                                                   t.lo[t.cur], t.id[t.cur], b.lo[out],
                                                                                   b.id[out], lowbits));
        }
    }
    cudaEventRecord(ev[3], st);
    unsigned long long ht[16] = {};
    MP_CUDA(cudaMemcpyAsync(ht, trace, sizeof ht, cudaMemcpyDeviceToHost, st));
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (stats) {
        float a = 0, bms = 0, c = 0;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&bms, ev[1], ev[2]);
        cudaEventElapsedTime(&c, ev[2], ev[3]);
        stats->tuples = n;
        stats->passes = (int)passes.size();
        stats->pass_ms = a;
        stats->bytes = (uint64_t)passes.size() * 2 * (12 + (has_hi ? 1 : 0)) * n;
        stats->seg_ms = bms;
        stats->big_ms = c;
        stats->units = nu + nm;
        stats->big_buckets = nb;
        stats->big_tuples = nbig;
        stats->unit_passes = ht[0];
        for (int q = 0; q < 3; q++) stats->phase_cycles[q] = ht[1 + q];
        for (int q = 0; q < 7; q++) stats->pass_cycles[q] = ht[8 + q];
    }
    arena.free_scratch(status);
    if (herr) return set_error(MP_EDEVICE, "radix sort look-back gave up (device error flags 0x%x)", herr);
    *out_lo_buf = out;  // lo and id end in the other buffer; hi (constant within a bucket) stays in `in`
    *out_hi_buf = in;
    b.cur = out;
    return 0;
}

// ---------------------------------------------------------------------------
// Allocation-free sort (mp_sort_tuples_noalloc).
//
// For callers that cannot allocate device memory once they are running -- a host that
// hands this library only pre-allocated buffers from its own allocator, or code that must
// not allocate inside a latency-critical loop -- the sort's scratch (the second tuple
// buffer, the look-back status words, the digit histograms) lives in one fixed device
// array declared here.  Every GPU that loads the library holds it (about 14 MB) until the
// process exits.  Calls share the array: two calls in flight at the same time on the GPU
// (different streams, or host threads) race on it and corrupt each other's results.
constexpr uint64_t NOALLOC_MAX_TUPLES = 1ull << 20;
constexpr uint64_t NOALLOC_TILES = (NOALLOC_MAX_TUPLES + STILE - 1) / STILE;

struct NoAllocScratch {
    uint64_t lo[NOALLOC_MAX_TUPLES];
    uint32_t id[NOALLOC_MAX_TUPLES];
    uint8_t hi[NOALLOC_MAX_TUPLES];
    unsigned long long status[NOALLOC_TILES * 256];
    unsigned long long ghist[9 * 256];
    uint64_t dbase[9 * 256];
    uint32_t ctr[16];
    uint32_t err;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device ordinal (host code cannot use the symbol
// itself: in host code it names a host-side shadow, not device memory).
static NoAllocScratch *g_noalloc_addr[256];
static std::mutex g_noalloc_mu;

static int noalloc_scratch(NoAllocScratch **out)
{
    int dev = 0;
    MP_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return set_error(MP_EUNSUP, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return set_cuda_error(e, "cudaGetSymbolAddress(scratch)", __FILE__, __LINE__);
        g_noalloc_addr[dev] = (NoAllocScratch *)p;
    }
    *out = g_noalloc_addr[dev];
    return 0;
}

// [a, a + an) and [b, b + bn) share a byte.
static bool bytes_overlap(const void *a, uint64_t an, const void *b, uint64_t bn)
{
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
    return an && bn && x < y + bn && y < x + an;
}

int sort_tuples_noalloc(const uint64_t *lo_in, const uint8_t *hi_in, const uint32_t *id_in, uint64_t *lo_out,
                        uint8_t *hi_out, uint32_t *id_out, uint64_t n, cudaStream_t st)
{
    if (!lo_in || !id_in || !lo_out || !id_out) return set_error(MP_EARG, "null argument");
    if ((hi_in == nullptr) != (hi_out == nullptr))
        return set_error(MP_EARG, "hi_in and hi_out must both be given or both NULL");
    if (n > NOALLOC_MAX_TUPLES)
        return set_error(MP_EARG, "%llu tuples exceed the fixed scratch of the allocation-free sort (%llu tuples)",
                         (unsigned long long)n, (unsigned long long)NOALLOC_MAX_TUPLES);
    const bool has_hi = hi_in != nullptr;
    // each output array is either the same array as its input (sorted in place) or apart from every input
    const void *ins[3] = {lo_in, id_in, hi_in};
    const uint64_t insz[3] = {n * 8, n * 4, has_hi ? n : 0};
    const void *outs[3] = {lo_out, id_out, hi_out};
    bool in_place = false;
    for (int o = 0; o < 3; o++)
        for (int i = 0; i < 3; i++) {
            if (!bytes_overlap(outs[o], insz[o], ins[i], insz[i])) continue;
            if (o != i || outs[o] != ins[i])
                return set_error(MP_EARG, "an output array overlaps an input array other than its own in-place input");
            in_place = true;
        }
    NoAllocScratch *S = nullptr;
    int rc = noalloc_scratch(&S);
    if (rc) return rc;
    if (n == 0) return 0;
    const uint64_t tiles = (n + STILE - 1) / STILE;
    // the array keeps the previous call's contents: clear what must start at zero
    MP_CUDA(cudaMemsetAsync(S->ghist, 0, sizeof S->ghist, st));
    MP_CUDA(cudaMemsetAsync(S->ctr, 0, sizeof S->ctr, st));
    MP_CUDA(cudaMemsetAsync(&S->err, 0, sizeof S->err, st));
    MP_CUDA(cudaMemsetAsync(S->status, 0, tiles * 256 * sizeof(unsigned long long), st));
    (mp::count_launch(), k_hist_upfront<<<2 * sm_count(), 256, 0, st>>>(lo_in, hi_in, n, S->ghist));
    unsigned long long h[9 * 256];
    MP_CUDA(cudaMemcpyAsync(h, S->ghist, sizeof h, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    int passes[9], np = 0;
    uint64_t base[9 * 256];
    for (int dgt = 0; dgt < (has_hi ? 9 : 8); dgt++) {
        uint64_t acc = 0;
        bool constant = false;
        for (int v = 0; v < 256; v++) {
            base[dgt * 256 + v] = acc;
            if (h[dgt * 256 + v] == n) constant = true;
            acc += h[dgt * 256 + v];
        }
        if (acc != n) return set_error(MP_EDEVICE, "radix histogram does not add up");
        if (!constant) passes[np++] = dgt;
    }
    if (np == 0) {  // every digit constant: the input is already in order (nothing to move in place)
        if (lo_out != lo_in) MP_CUDA(cudaMemcpyAsync(lo_out, lo_in, n * 8, cudaMemcpyDeviceToDevice, st));
        if (id_out != id_in) MP_CUDA(cudaMemcpyAsync(id_out, id_in, n * 4, cudaMemcpyDeviceToDevice, st));
        if (has_hi && hi_out != hi_in) MP_CUDA(cudaMemcpyAsync(hi_out, hi_in, n, cudaMemcpyDeviceToDevice, st));
        MP_CUDA(cudaStreamSynchronize(st));
        return 0;
    }
    MP_CUDA(cudaMemcpyAsync(S->dbase, base, sizeof base, cudaMemcpyHostToDevice, st));
    sort_kernel_attrs();
    // pass i writes the caller's output when (np - 1 - i) is even, the scratch otherwise, so the last
    // pass always lands in the output.  A pass must not write the array it reads: in place with an odd
    // pass count, pass 0 would, so the input is first copied to the scratch and pass 0 reads it there.
    const uint64_t *src_lo = lo_in;
    const uint8_t *src_hi = hi_in;
    const uint32_t *src_id = id_in;
    if (in_place && (np & 1)) {
        MP_CUDA(cudaMemcpyAsync(S->lo, lo_in, n * 8, cudaMemcpyDeviceToDevice, st));
        MP_CUDA(cudaMemcpyAsync(S->id, id_in, n * 4, cudaMemcpyDeviceToDevice, st));
        if (has_hi) MP_CUDA(cudaMemcpyAsync(S->hi, hi_in, n, cudaMemcpyDeviceToDevice, st));
        src_lo = S->lo;
        src_id = S->id;
        src_hi = has_hi ? S->hi : nullptr;
    }
    for (int i = 0; i < np; i++) {
        const bool to_out = ((np - 1 - i) & 1) == 0;
        uint64_t *d_lo = to_out ? lo_out : S->lo;
        uint32_t *d_id = to_out ? id_out : S->id;
        uint8_t *d_hi = has_hi ? (to_out ? hi_out : S->hi) : nullptr;
        const int dgt = passes[i];
        if (dgt < 8)
            (mp::count_launch(), k_onesweep<0><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(
                src_lo, src_hi, src_id, d_lo, d_hi, d_id, n, 8 * dgt, 8, S->dbase + dgt * 256, nullptr, S->status, S->ctr + i,
                (uint32_t)(i + 1), &S->err, 0u, nullptr, Segs{}, WaitLimits{}.lookback_spins));
        else
            (mp::count_launch(), k_onesweep<1><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(
                src_lo, src_hi, src_id, d_lo, d_hi, d_id, n, 0, 8, S->dbase + dgt * 256, nullptr, S->status, S->ctr + i,
                (uint32_t)(i + 1), &S->err, 0u, nullptr, Segs{}, WaitLimits{}.lookback_spins));
        src_lo = d_lo;
        src_hi = d_hi;
        src_id = d_id;
    }
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(&herr, &S->err, sizeof herr, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (herr) return set_error(MP_EDEVICE, "radix sort look-back gave up (device error flags 0x%x)", herr);
    return 0;
}

}  // namespace mp

extern "C" int mp_sort_tuples_noalloc(const uint64_t *lo_in, const uint8_t *hi_in, const uint32_t *id_in,
                                      uint64_t *lo_out, uint8_t *hi_out, uint32_t *id_out, uint64_t n, void *stream)
{
    return mp::sort_tuples_noalloc(lo_in, hi_in, id_in, lo_out, hi_out, id_out, n, (cudaStream_t)stream);
}
