// K0: FASTQ parsing on the GPU, plus the device-wide exclusive scans every stage uses.
//
// A record is four '\n'-terminated lines (header, sequence, '+', quality) with the
// quality as long as the sequence -- the walk getNextRead does (genHistograms.c:60-80,
// metapart.c:296-369).  The parser finds every newline with coalesced 16-byte loads,
// compacts their positions in order, and derives the record table from every fourth one.
#include <cstdio>

#include "k_reads.cuh"

namespace mp {

// ------------------------------------------------------------------ scans

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ uint64_t load_or_zero(const T *in, uint64_t i, uint64_t n)
{
    return i < n ? (uint64_t)in[i] : 0ull;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix, *total = block sum.
__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t *total)
{
    __shared__ uint64_t warp_sums[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint64_t w = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    uint64_t before = wid ? warp_sums[wid - 1] : 0;
    *total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_sums(const T *in, uint64_t n, uint64_t *sums)
{
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint64_t s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) s += load_or_zero(in, base + (uint64_t)j * SCAN_THREADS + threadIdx.x, n);
    uint64_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_scan(const T *in, uint64_t *out, uint64_t n,
                                                            const uint64_t *offsets, uint64_t *total)
{
    __shared__ uint64_t tile[SCAN_TILE];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        int idx = j * SCAN_THREADS + threadIdx.x;
        tile[idx] = load_or_zero(in, base + idx, n);
    }
    __syncthreads();
    uint64_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) { v[j] = tile[threadIdx.x * SCAN_ITEMS + j]; s += v[j]; }
    uint64_t tot;
    uint64_t run = block_excl_scan(s, &tot) + (offsets ? offsets[blockIdx.x] : 0ull);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) { tile[threadIdx.x * SCAN_ITEMS + j] = run; run += v[j]; }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        int idx = j * SCAN_THREADS + threadIdx.x;
        if (base + idx < n) out[base + idx] = tile[idx];
    }
    if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_THREADS - 1) *total = run;
}

size_t scan_tmp_bytes(uint64_t n)
{
    size_t b = 0;
    while (n > (uint64_t)SCAN_TILE) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        b += n * sizeof(uint64_t) + 256;
    }
    return b + 256;
}

template <typename T>
static void scan_impl(const T *in, uint64_t *out, uint64_t n, uint64_t *total_dev, void *tmp, size_t tmp_bytes,
                      cudaStream_t st)
{
    if (n == 0) {
        if (total_dev) cudaMemsetAsync(total_dev, 0, sizeof(uint64_t), st);
        return;
    }
    uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        (mp::count_launch(), k_tile_scan<T><<<1, SCAN_THREADS, 0, st>>>(in, out, n, nullptr, total_dev));
        return;
    }
    uint64_t *sums = (uint64_t *)tmp;
    size_t used = (tiles * sizeof(uint64_t) + 255) & ~(size_t)255;
    (mp::count_launch(), k_tile_sums<T><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, n, sums));
    scan_impl<uint64_t>(sums, sums, tiles, nullptr, (char *)tmp + used, tmp_bytes - used, st);
    (mp::count_launch(), k_tile_scan<T><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, out, n, sums, total_dev));
}

void scan_u32_to_u64(const uint32_t *in, uint64_t *out, uint64_t n, uint64_t *total_dev, void *tmp,
                     size_t tmp_bytes, cudaStream_t st)
{
    scan_impl<uint32_t>(in, out, n, total_dev, tmp, tmp_bytes, st);
}
void scan_u64(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t *total_dev, void *tmp, size_t tmp_bytes,
              cudaStream_t st)
{
    scan_impl<uint64_t>(in, out, n, total_dev, tmp, tmp_bytes, st);
}

// ---------------------------------------------------------------- newlines

constexpr int NL_THREADS = 256;
constexpr uint64_t NL_SEG = 65536;  // bytes per block; a multiple of 16 * NL_THREADS

__device__ __forceinline__ uint32_t nl_in_word(uint32_t w)
{
    // 0x80 in exactly the bytes equal to '\n' (0x0A): exact zero-byte test of w ^ 0x0A0A0A0A
    // (no carry crosses a byte: (x & 0x7F) + 0x7F <= 0xFE)
    const uint32_t x = w ^ 0x0A0A0A0Au;
    const uint32_t y = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
    return ~(y | x | 0x7F7F7F7Fu);
}

// buf is 16-byte aligned; its first `skip` (< 16) bytes are not part of the parsed range, whose byte 0 is
// buf[skip] (newline positions are written relative to it).
__global__ void __launch_bounds__(NL_THREADS) k_nl_count(const uint8_t *buf, uint64_t n, uint32_t skip, uint32_t *seg_counts)
{
    const uint64_t s0 = (uint64_t)blockIdx.x * NL_SEG, s1 = min(n, s0 + NL_SEG);
    uint32_t c = 0;
    for (uint64_t p = s0 + (uint64_t)threadIdx.x * 16; p < s1; p += NL_THREADS * 16) {
        if (p + 16 <= s1 && p >= skip) {
            uint4 v = *reinterpret_cast<const uint4 *>(buf + p);
            c += __popc(nl_in_word(v.x)) + __popc(nl_in_word(v.y)) + __popc(nl_in_word(v.z)) + __popc(nl_in_word(v.w));
        } else {
            for (uint64_t q = max(p, (uint64_t)skip); q < min(s1, p + 16); q++) c += buf[q] == '\n';
        }
    }
    uint64_t tot;
    uint64_t x = c;
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
    __shared__ uint64_t ws[NL_THREADS / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        tot = 0;
        for (int w = 0; w < NL_THREADS / 32; w++) tot += ws[w];
        seg_counts[blockIdx.x] = (uint32_t)tot;
    }
}

__global__ void __launch_bounds__(NL_THREADS) k_nl_write(const uint8_t *buf, uint64_t n, uint32_t skip,
                                                         const uint64_t *seg_off, uint64_t *nl_pos)
{
    const uint64_t s0 = (uint64_t)blockIdx.x * NL_SEG, s1 = min(n, s0 + NL_SEG);
    uint64_t out = seg_off[blockIdx.x];
    for (uint64_t r = s0; r < s1; r += NL_THREADS * 16) {
        const uint64_t p = r + (uint64_t)threadIdx.x * 16;
        uint8_t b[16];
        int cnt = 0;
        if (p + 16 <= s1 && p >= skip) {
            uint4 v = *reinterpret_cast<const uint4 *>(buf + p);
            memcpy(b, &v, 16);
            cnt = __popc(nl_in_word(v.x)) + __popc(nl_in_word(v.y)) + __popc(nl_in_word(v.z)) + __popc(nl_in_word(v.w));
        } else {
            for (int q = 0; q < 16; q++) {
                b[q] = (p + q < s1 && p + q >= skip) ? buf[p + q] : 0;
                cnt += b[q] == '\n';
            }
        }
        uint64_t tot;
        uint64_t pre = block_excl_scan((uint64_t)cnt, &tot);
        uint64_t o = out + pre;
#pragma unroll
        for (int q = 0; q < 16; q++)
            if (b[q] == '\n') nl_pos[o++] = p + q - skip;
        out += tot;
    }
}

// Record table from the newline positions; flags quality/sequence length mismatches.
__global__ void k_records(const uint64_t *nl, uint64_t n_rec, uint64_t *rec_start, uint64_t *seq_off, uint32_t *seq_len,
                          unsigned long long *first_bad)
{
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rec) return;
    uint64_t s = r ? nl[4 * r - 1] + 1 : 0;
    uint64_t sq = nl[4 * r] + 1;
    uint64_t sl = nl[4 * r + 1] - sq;
    uint64_t q = nl[4 * r + 2] + 1;
    uint64_t ql = nl[4 * r + 3] - q;
    rec_start[r] = s;
    seq_off[r] = sq;
    seq_len[r] = (uint32_t)sl;
    if (ql != sl || sl > 0xFFFFFFFFull) atomicMin(first_bad, (unsigned long long)r);
    if (r == n_rec - 1) rec_start[n_rec] = nl[4 * r + 3] + 1;
}

// For each query offset: the record whose start equals it, or ~0 when no record starts there.
__global__ void k_record_of_offset(const uint64_t *rec_start, uint64_t n_rec, const uint64_t *queries, int nq,
                                   uint64_t *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    uint64_t x = queries[i], lo = 0, hi = n_rec + 1;  // search rec_start[0..n_rec]
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (rec_start[mid] < x) lo = mid + 1; else hi = mid;
    }
    out[i] = (lo <= n_rec && rec_start[lo] == x) ? lo : ~0ull;
}

int parse_fastq(const uint8_t *d_buf, uint64_t n, ParsedReads *pr, DeviceArena &arena, cudaStream_t st)
{
    return parse_fastq_range(d_buf, 0, n, pr, arena, st);
}

int parse_fastq_range(const uint8_t *d_base, uint64_t begin, uint64_t end, ParsedReads *pr, DeviceArena &arena,
                      cudaStream_t st)
{
    const uint64_t n = end - begin;
    if (n == 0 || end < begin) return set_error(MP_EFMT, "empty FASTQ input");
    // the kernels read 16-byte words from the 16-byte boundary at or below begin and skip the bytes before it
    const uint64_t a0 = begin & ~15ull;
    const uint32_t skip = (uint32_t)(begin - a0);
    const uint8_t *d_buf = d_base + a0;
    const uint64_t na = end - a0;
    const uint64_t segs = (na + NL_SEG - 1) / NL_SEG;
    uint32_t *seg_counts = arena.alloc<uint32_t>(segs);
    uint64_t *seg_off = arena.alloc<uint64_t>(segs + 1);
    uint64_t *total = arena.alloc<uint64_t>(1);
    size_t tb = scan_tmp_bytes(segs);
    void *tmp = arena.alloc<uint8_t>(tb);
    if (!seg_counts || !seg_off || !total || !tmp) return set_error(MP_ENOMEM, "device memory for the FASTQ parse");
    (mp::count_launch(), k_nl_count<<<(unsigned)segs, NL_THREADS, 0, st>>>(d_buf, na, skip, seg_counts));
    scan_u32_to_u64(seg_counts, seg_off, segs, total, tmp, tb, st);
    uint64_t n_nl = 0;
    MP_CUDA(cudaMemcpyAsync(&n_nl, total, sizeof n_nl, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    if (n_nl == 0 || n_nl % 4) return set_error(MP_EFMT, "FASTQ line count %llu is not a multiple of 4", (unsigned long long)n_nl);
    uint64_t *nl = arena.alloc<uint64_t>(n_nl);
    if (!nl) return set_error(MP_ENOMEM, "device memory for newline positions");
    (mp::count_launch(), k_nl_write<<<(unsigned)segs, NL_THREADS, 0, st>>>(d_buf, na, skip, seg_off, nl));
    const uint64_t n_rec = n_nl / 4;
    pr->n_reads = n_rec;
    pr->rec_start = arena.alloc_persistent<uint64_t>(n_rec + 1);
    pr->seq_off = arena.alloc_persistent<uint64_t>(n_rec);
    pr->seq_len = arena.alloc_persistent<uint32_t>(n_rec);
    unsigned long long *bad = arena.alloc<unsigned long long>(1);
    if (!pr->rec_start || !pr->seq_off || !pr->seq_len || !bad) return set_error(MP_ENOMEM, "device memory for the record table");
    MP_CUDA(cudaMemsetAsync(bad, 0xFF, sizeof *bad, st));
    (mp::count_launch(), k_records<<<(unsigned)((n_rec + 255) / 256), 256, 0, st>>>(nl, n_rec, pr->rec_start, pr->seq_off, pr->seq_len, bad));
    unsigned long long hb = 0;
    uint64_t last_end = 0;
    MP_CUDA(cudaMemcpyAsync(&hb, bad, sizeof hb, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaMemcpyAsync(&last_end, pr->rec_start + n_rec, sizeof last_end, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    if (hb != ~0ull) return set_error(MP_EFMT, "FASTQ record %llu: quality length differs from the sequence length", hb);
    if (last_end != n) return set_error(MP_EFMT, "FASTQ input does not end with a complete record");
    arena.release_scratch();
    return 0;
}

// Record table of one input segment (offsets relative to the segment) into the job's table at read r0,
// offsets moved by the segment's byte offset; n + 1 start entries (the last is the next segment's first).
__global__ void k_concat_records(const uint64_t *rs, const uint64_t *so, const uint32_t *sl, uint64_t n, uint64_t base,
                                 uint64_t *drs, uint64_t *dso, uint32_t *dsl)
{
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r > n) return;
    drs[r] = rs[r] + base;
    if (r < n) {
        dso[r] = so[r] + base;
        dsl[r] = sl[r];
    }
}

void concat_records(const ParsedReads &seg, uint64_t byte_base, ParsedReads &dst, uint64_t r0, cudaStream_t st)
{
    (mp::count_launch(), k_concat_records<<<(unsigned)((seg.n_reads + 1 + 255) / 256), 256, 0, st>>>(
        seg.rec_start, seg.seq_off, seg.seq_len, seg.n_reads, byte_base, dst.rec_start + r0, dst.seq_off + r0,
        dst.seq_len + r0));
}

int records_at_offsets(const ParsedReads *pr, const uint64_t *h_offsets, int nq, uint64_t *h_rec, DeviceArena &arena,
                       cudaStream_t st)
{
    uint64_t *dq = arena.alloc<uint64_t>(nq), *dr = arena.alloc<uint64_t>(nq);
    if (!dq || !dr) return set_error(MP_ENOMEM, "device memory");
    MP_CUDA(cudaMemcpyAsync(dq, h_offsets, nq * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    (mp::count_launch(), k_record_of_offset<<<(nq + 127) / 128, 128, 0, st>>>(pr->rec_start, pr->n_reads, dq, nq, dr));
    MP_CUDA(cudaMemcpyAsync(h_rec, dr, nq * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    arena.release_scratch();
    for (int i = 0; i < nq; i++)
        if (h_rec[i] == ~0ull)
            return set_error(MP_EFMT, "offset %llu is not the start of a FASTQ record", (unsigned long long)h_offsets[i]);
    return 0;
}

}  // namespace mp
