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
#include <cstdio>
#include <mutex>
#include <vector>

#include "k_sort.cuh"

namespace mp {

constexpr int ST = 256;
constexpr int SI = 16;
constexpr int STILE = ST * SI;
constexpr int SW = ST / 32;
constexpr unsigned FULLM = 0xFFFFFFFFu;
constexpr uint32_t SPIN_CAP = 1u << 22;

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
};

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

template <int SRC>
__global__ void __launch_bounds__(ST) k_onesweep(const uint64_t *__restrict__ in_lo, const uint8_t *__restrict__ in_hi,
                                                 const uint32_t *__restrict__ in_id, uint64_t *__restrict__ out_lo,
                                                 uint8_t *__restrict__ out_hi, uint32_t *__restrict__ out_id, uint64_t n,
                                                 int shift, const uint64_t *__restrict__ dbase,
                                                 unsigned long long *status, uint32_t *tile_ctr, uint32_t epoch,
                                                 uint32_t *err)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    SortSmem &sm = *reinterpret_cast<SortSmem *>(smraw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < SW * 256; i += ST) (&sm.whist[0][0])[i] = 0;
    if (threadIdx.x == 0) sm.tile_id = atomicAdd(tile_ctr, 1u);
    __syncthreads();
    const uint64_t tile = sm.tile_id;
    const uint64_t base = tile * STILE;
    const bool has_hi = in_hi != nullptr;

    uint64_t key[SI];
    uint32_t val[SI], rank[SI], dg[SI];
    uint8_t hv[SI];
#pragma unroll
    for (int j = 0; j < SI; j++) {
        const uint64_t idx = base + (uint64_t)warp * (32 * SI) + (uint64_t)j * 32 + lane;
        const bool v = idx < n;
        key[j] = v ? in_lo[idx] : 0ull;
        val[j] = v ? in_id[idx] : 0u;
        hv[j] = (has_hi && v) ? in_hi[idx] : (uint8_t)0;
        dg[j] = v ? (SRC == 0 ? (uint32_t)((key[j] >> shift) & 0xFF) : (uint32_t)hv[j]) : 256u;
    }
    // warp-level multi-split: stable rank of each tuple among equal digits of its warp
    const uint32_t lt = (1u << lane) - 1;
#pragma unroll
    for (int j = 0; j < SI; j++) {
        const uint32_t d = dg[j];
        const uint32_t peers = __match_any_sync(FULLM, d);
        uint32_t pre = 0;
        if (d < 256) pre = sm.whist[warp][d];
        __syncwarp();
        if (d < 256) {
            rank[j] = pre + __popc(peers & lt);
            if ((peers & lt) == 0) sm.whist[warp][d] = pre + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // thread d: warp prefixes and tile count of digit d
    const uint32_t d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < SW; w++) {
        const uint32_t t = sm.whist[w][d];
        sm.whist[w][d] = run;
        run += t;
    }
    const uint32_t cnt = run;
    const unsigned long long E = (unsigned long long)epoch << 60, PF = 1ull << 59, CM = PF - 1;
    unsigned long long *me = status + tile * 256 + d;
    st_relaxed(me, tile == 0 ? (E | PF | cnt) : (E | cnt));
    // tile-local exclusive scan of digit counts
    {
        uint32_t x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(FULLM, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sm.wsum[warp] = x;
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; w++) before += sm.wsum[w];
        sm.tstart[d] = before + x - cnt;
    }
    // decoupled look-back for digit d
    unsigned long long excl = 0;
    if (tile > 0) {
        int64_t p = (int64_t)tile - 1;
        uint32_t spins = 0;
        while (p >= 0) {
            const unsigned long long v = ld_relaxed(status + (uint64_t)p * 256 + d);
            if ((v >> 60) != epoch) {
                if (++spins > SPIN_CAP) {
                    atomicOr(err, DERR_SPIN);
                    break;
                }
                continue;
            }
            excl += v & CM;
            if (v & PF) break;
            p--;
        }
        st_relaxed(me, E | PF | (excl + cnt));
    }
    sm.gbase[d] = dbase[d] + excl;
    if (threadIdx.x == 0) sm.nvalid = (uint32_t)min((uint64_t)STILE, n - base);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SI; j++) {
        if (dg[j] < 256) {
            const uint32_t s = sm.tstart[dg[j]] + sm.whist[warp][dg[j]] + rank[j];
            sm.keys[s] = key[j];
            sm.vals[s] = val[j];
            if (has_hi) sm.his[s] = hv[j];
        }
    }
    __syncthreads();
    const uint32_t nv = sm.nvalid;
    for (uint32_t s = threadIdx.x; s < nv; s += ST) {
        const uint64_t kk = sm.keys[s];
        const uint32_t dd = SRC == 0 ? (uint32_t)((kk >> shift) & 0xFF) : (uint32_t)sm.his[s];
        const uint64_t g = sm.gbase[dd] + (s - sm.tstart[dd]);
        if (g >= n) continue;  // only after a failed look-back (err is set)
        out_lo[g] = kk;
        out_id[g] = sm.vals[s];
        if (has_hi) out_hi[g] = sm.his[s];
    }
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
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    (mp::count_launch(), k_hist_upfront<<<152 * 8, 256, 0, st>>>(b.lo[b.cur], has_hi ? b.hi[b.cur] : nullptr, n, ghist));
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
        if (acc != n) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return set_error(MP_EDEVICE, "radix histogram does not add up");
        }
        if (!constant) passes.push_back(dgt);
    }
    MP_CUDA(cudaMemcpyAsync(dbase, base.data(), base.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_onesweep<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        cudaFuncSetAttribute(k_onesweep<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
        attr_set = true;
    }
    std::vector<cudaEvent_t> ev(passes.size() + 1);
    for (auto &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], st);
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const int dgt = passes[pi];
        const int src = b.cur, dst = b.cur ^ 1;
        const uint8_t *ih = has_hi ? b.hi[src] : nullptr;
        uint8_t *oh = has_hi ? b.hi[dst] : nullptr;
        if (dgt < 8)
            (mp::count_launch(), k_onesweep<0><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(b.lo[src], ih, b.id[src], b.lo[dst], oh,
                                                                         b.id[dst], n, 8 * dgt, dbase + dgt * 256, status,
                                                                         ctr + pi, (uint32_t)(pi + 1), err));
        else
            (mp::count_launch(), k_onesweep<1><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(b.lo[src], ih, b.id[src], b.lo[dst], oh,
                                                                         b.id[dst], n, 0, dbase + dgt * 256, status,
                                                                         ctr + pi, (uint32_t)(pi + 1), err));
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
    for (auto &e : ev) cudaEventDestroy(e);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    arena.free_scratch(status);
    if (herr) return set_error(MP_EDEVICE, "radix sort look-back gave up (device error flags 0x%x)", herr);
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

int sort_tuples_noalloc(const uint64_t *lo_in, const uint8_t *hi_in, const uint32_t *id_in, uint64_t *lo_out,
                        uint8_t *hi_out, uint32_t *id_out, uint64_t n, cudaStream_t st)
{
    if (!lo_in || !id_in || !lo_out || !id_out) return set_error(MP_EARG, "null argument");
    if ((hi_in == nullptr) != (hi_out == nullptr))
        return set_error(MP_EARG, "hi_in and hi_out must both be given or both NULL");
    if (n > NOALLOC_MAX_TUPLES)
        return set_error(MP_EARG, "%llu tuples exceed the fixed scratch of the allocation-free sort (%llu tuples)",
                         (unsigned long long)n, (unsigned long long)NOALLOC_MAX_TUPLES);
    NoAllocScratch *S = nullptr;
    int rc = noalloc_scratch(&S);
    if (rc) return rc;
    const bool has_hi = hi_in != nullptr;
    if (n == 0) return 0;
    const uint64_t tiles = (n + STILE - 1) / STILE;
    // the array keeps the previous call's contents: clear what must start at zero
    MP_CUDA(cudaMemsetAsync(S->ghist, 0, sizeof S->ghist, st));
    MP_CUDA(cudaMemsetAsync(S->ctr, 0, sizeof S->ctr, st));
    MP_CUDA(cudaMemsetAsync(&S->err, 0, sizeof S->err, st));
    MP_CUDA(cudaMemsetAsync(S->status, 0, tiles * 256 * sizeof(unsigned long long), st));
    (mp::count_launch(), k_hist_upfront<<<152 * 2, 256, 0, st>>>(lo_in, hi_in, n, S->ghist));
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
    if (np == 0) {  // every digit constant: the input is already in order
        MP_CUDA(cudaMemcpyAsync(lo_out, lo_in, n * 8, cudaMemcpyDeviceToDevice, st));
        MP_CUDA(cudaMemcpyAsync(id_out, id_in, n * 4, cudaMemcpyDeviceToDevice, st));
        if (has_hi) MP_CUDA(cudaMemcpyAsync(hi_out, hi_in, n, cudaMemcpyDeviceToDevice, st));
        MP_CUDA(cudaStreamSynchronize(st));
        return 0;
    }
    MP_CUDA(cudaMemcpyAsync(S->dbase, base, sizeof base, cudaMemcpyHostToDevice, st));
    static bool attr = false;
    if (!attr) {
        MP_CUDA(cudaFuncSetAttribute(k_onesweep<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem)));
        MP_CUDA(cudaFuncSetAttribute(k_onesweep<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem)));
        attr = true;
    }
    // pass i writes the caller's output when (np - 1 - i) is even, the scratch otherwise,
    // so the last pass always lands in the output
    const uint64_t *src_lo = lo_in;
    const uint8_t *src_hi = hi_in;
    const uint32_t *src_id = id_in;
    for (int i = 0; i < np; i++) {
        const bool to_out = ((np - 1 - i) & 1) == 0;
        uint64_t *d_lo = to_out ? lo_out : S->lo;
        uint32_t *d_id = to_out ? id_out : S->id;
        uint8_t *d_hi = has_hi ? (to_out ? hi_out : S->hi) : nullptr;
        const int dgt = passes[i];
        if (dgt < 8)
            (mp::count_launch(), k_onesweep<0><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(
                src_lo, src_hi, src_id, d_lo, d_hi, d_id, n, 8 * dgt, S->dbase + dgt * 256, S->status, S->ctr + i,
                (uint32_t)(i + 1), &S->err));
        else
            (mp::count_launch(), k_onesweep<1><<<(unsigned)tiles, ST, sizeof(SortSmem), st>>>(
                src_lo, src_hi, src_id, d_lo, d_hi, d_id, n, 0, S->dbase + dgt * 256, S->status, S->ctr + i,
                (uint32_t)(i + 1), &S->err));
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
