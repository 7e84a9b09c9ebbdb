// K1 (m-mer histogram) and K2 (tuple enumeration) kernels.
//
// Plain variant: one warp per read.  Each round of 32 bases is loaded with one
// coalesced byte load per lane; two warp OR-reductions pack the 2-bit base codes
// most-significant-first into a 64-bit word and a ballot gives the N mask.  Lane j
// of round t then owns k-mer position 32t+j: its forward code is a funnel shift of
// two packed words, its reverse complement a bit reversal, and the neighbouring
// characters of the adjacency byte come by shuffle (countMmers.c:83-217,
// enumerateKmers.c:127-371 compute the same codes with a rolling update).
//
// 3-minimizer variant: one thread per read running the reference's window logic
// (countMmers_3minimizers.c:83-271, enumerateKmers_3minimizers.c:129-470); it
// emits about three k-mers per read, so the base scan dominates either way.
#include "k_kmers.cuh"

namespace mp {

constexpr unsigned FULL = 0xFFFFFFFFu;

struct Round {
    uint64_t W;  // codes of positions 32t..32t+31, position 32t in bits 63..62
    uint32_t N;  // bit j: position 32t+j is 'N'
    uint32_t c;  // this lane's character (position 32t+lane); the adjacency bytes take neighbours by shuffle
};

__device__ __forceinline__ void load_round(const uint8_t *s, uint32_t L, int t, int lane, Round &r)
{
    const uint32_t p = 32u * (uint32_t)t + (uint32_t)lane;
    const uint32_t c = p < L ? (uint32_t)s[p] : 0x41u;
    // lane j's code goes to bits 63-2j..62-2j of W: two warp OR-reductions build the halves
    const uint32_t f = fcode(c) << (30 - 2 * (lane & 15));
    const uint32_t hi = __reduce_or_sync(FULL, lane < 16 ? f : 0u), lo = __reduce_or_sync(FULL, lane < 16 ? 0u : f);
    r.W = ((uint64_t)hi << 32) | lo;
    r.N = __ballot_sync(FULL, p < L && c == 'N');
    r.c = c;
}

// The same round from the 2-bit packed reads: one 64-bit code word and one 32-bit N mask per 32 bases,
// as load_round builds them (positions past the read are code 0 and not N); the lane's character is
// restored from its code (ACGT) or the mask (N), which is exact for reads of those five letters only
// (the count pass stores no packed copy of an input with any other byte).
__device__ __forceinline__ void load_round_packed(const uint64_t *w, const uint32_t *nm, uint32_t nrounds, int t, int lane,
                                                  Round &r)
{
    const bool in = (uint32_t)t < nrounds;
    r.W = in ? w[t] : 0ull;
    r.N = in ? nm[t] : 0u;
    const uint32_t code = (uint32_t)(r.W >> (62 - 2 * lane)) & 3u;
    r.c = ((r.N >> lane) & 1u) ? 0x4Eu : ((0x54474341u >> (8 * code)) & 0xFFu);  // N, or A C G T
}

// Forward code, validity (no N in the window) of the k-mer at lane's position of round t.
__device__ __forceinline__ bool kmer_at(int lane, int k, const Round &c, const Round &n, uint64_t &fwd)
{
    const uint64_t x = lane ? ((c.W << (2 * lane)) | (n.W >> (64 - 2 * lane))) : c.W;
    fwd = x >> (64 - 2 * k);
    const uint64_t n64 = (uint64_t)c.N | ((uint64_t)n.N << 32);
    return ((n64 >> lane) & ((1ull << k) - 1)) == 0;
}

__device__ __forceinline__ uint32_t chunk_of(const uint64_t *chunk_rec, int nchunks, uint64_t r)
{
    int lo = 0, hi = nchunks - 1;  // largest c with chunk_rec[c] <= r
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (chunk_rec[mid] <= r) lo = mid; else hi = mid - 1;
    }
    return (uint32_t)lo;
}

// ------------------------------------------------------------ K1 plain

// KC: per position of every read, lo = canon << 8 | adj and hi = canon >> 56, or hi = KC_NONE
// when the window holds an N.  Written by the count pass when kc_lo is given; the partition's
// scans then filter this array instead of recomputing k-mers.
constexpr uint8_t KC_NONE = 0xFF;
constexpr int KC_PER_LANE = 10;  // cached positions per lane of a read: L - k + 1 <= 300

// PK: the read's rounds also go to the packed copy at pk_off[r] (ceil(L / 32) rounds of a code word and an
// N mask); a byte other than A, C, G, T, N sets DERR_NONACGT (no packed copy is usable).
template <bool PK>
__global__ void __launch_bounds__(256) k_count_plain(const uint8_t *fq, const uint64_t *seq_off, const uint32_t *seq_len,
                                                     uint64_t r0, uint64_t r1, int k, const uint64_t *chunk_rec,
                                                     int nchunks, uint32_t *cc, unsigned long long *glob, uint32_t *err,
                                                     const uint64_t *kc_off, uint64_t *kc_lo, uint8_t *kc_hi,
                                                     const uint64_t *pk_off, uint64_t *pk_w, uint32_t *pk_n)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int sh = 2 * (k - 10);
    for (uint64_t r = r0 + (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < r1; r += nw) {
        const uint32_t L = seq_len[r];
        if (L <= (uint32_t)k) continue;
        if (L > (uint32_t)MAX_READ_COUNT) {
            if (lane == 0) atomicOr(err, DERR_LONG_READ);
            continue;
        }
        const uint8_t *s = fq + seq_off[r];
        uint32_t *ccc = cc ? cc + (size_t)chunk_of(chunk_rec, nchunks, r) * NB : nullptr;
        const int last = (int)L - k;
        const uint64_t kbase = kc_lo ? kc_off[r] : 0;
        Round prv, cur, nxt;
        load_round(s, L, 0, lane, cur);
        load_round(s, L, 1, lane, nxt);
        prv = cur;
        const uint64_t pbase = PK ? pk_off[r] : 0;
        const uint32_t nrounds = (L + 31) / 32;
        int t = 0;
        for (; 32 * t <= last; t++) {
            const int i = 32 * t + lane;
            uint64_t fwd;
            bool v = kmer_at(lane, k, cur, nxt, fwd) && i <= last;
            const uint64_t rc = revcomp(fwd, k);
            const bool f = fwd < rc;
            const uint64_t canon = f ? fwd : rc;
            const uint32_t b = (uint32_t)(canon >> sh);
            if constexpr (PK) {  // the packed copy of round t
                const uint32_t c = cur.c;
                const bool odd = (uint32_t)(32 * t + lane) < L && c != 'A' && c != 'C' && c != 'G' && c != 'T' && c != 'N';
                if (__any_sync(FULL, odd) && lane == 0) atomicOr(err, DERR_NONACGT);
                if (lane == 0 && (uint32_t)t < nrounds) {
                    pk_w[pbase + t] = cur.W;
                    pk_n[pbase + t] = cur.N;
                }
            }
            if (kc_lo) {
                const uint32_t x = __shfl_sync(FULL, cur.c, (lane + 31) & 31), y = __shfl_sync(FULL, prv.c, 31);
                const int q = lane + k;
                const uint32_t u = __shfl_sync(FULL, cur.c, q & 31), w = __shfl_sync(FULL, nxt.c, q & 31);
                if (i <= last) {
                    // 'N' at the read ends (enumerateKmers.c:177, 252-255)
                    const uint32_t pa = i > 0 ? a5_of(lane ? x : y) : 7u, na = i < last ? a5_of(q < 32 ? u : w) : 7u;
                    const uint32_t adj = f ? adj_fwd(pa, na) : adj_rc(pa, na);
                    kc_lo[kbase + i] = (canon << 8) | adj;
                    kc_hi[kbase + i] = v ? (uint8_t)(canon >> 56) : KC_NONE;
                }
            }
            // one reduction per k-mer: neighbouring positions almost never share a bucket, so grouping
            // equal buckets within the warp first costs more than it saves
            if (v) {
                if (ccc) atomicAdd(&ccc[b], 1u);
                else atomicAdd(&glob[b], 1ull);
            }
            prv = cur;
            cur = nxt;
            load_round(s, L, t + 2, lane, nxt);
        }
        if constexpr (PK) {  // the rounds after the last k-mer's (at most one: L < 32 t + 32 once 32 t > L - k, k < 32)
            for (; (uint32_t)t < nrounds; t++) {
                const uint32_t c = cur.c;
                const bool odd = (uint32_t)(32 * t + lane) < L && c != 'A' && c != 'C' && c != 'G' && c != 'T' && c != 'N';
                if (__any_sync(FULL, odd) && lane == 0) atomicOr(err, DERR_NONACGT);
                if (lane == 0) {
                    pk_w[pbase + t] = cur.W;
                    pk_n[pbase + t] = cur.N;
                }
                cur = nxt;
                load_round(s, L, t + 2, lane, nxt);
            }
        }
    }
}

// Rounds of 32 bases per read for the packed copy (ceil(L / 32) when the read has a k-mer, else 0).
__global__ void k_pk_rounds(const uint32_t *seq_len, uint64_t n, int k, uint32_t *nr)
{
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) nr[r] = seq_len[r] > (uint32_t)k ? (seq_len[r] + 31) / 32 : 0u;
}

// Positions per read (L - k + 1, or 0), for the k-mer cache offsets.
__global__ void k_kc_positions(const uint32_t *seq_len, uint64_t n, int k, uint32_t *npos)
{
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) npos[r] = seq_len[r] > (uint32_t)k ? seq_len[r] - (uint32_t)k + 1 : 0u;
}

// ------------------------------------------------------- 3-minimizer core

// One read, thread-sequential.  ENUM: apply the scan range and produce adjacency bytes.
template <bool ENUM, class Emit>
__device__ __forceinline__ void min3_read(const uint8_t *s, int L, int k, uint32_t lo, uint32_t hi, Emit emit)
{
    if (L <= k) return;
    const int last = L - k, sh = 2 * (k - 10), win = last / 3;
    const uint64_t mask = kmer_mask(k);
    uint64_t fwd = 0, rc = 0, mn = 0;
    uint32_t mps = 0, mns = 0;  // stored adjacency a5 values of the current minimum
    int lastN = -1;
    for (int j = 0; j < k; j++) {
        const uint32_t c = s[j];
        if (c == 'N') lastN = j;
        rc |= (uint64_t)(3u - fcode(c)) << (2 * j);
        fwd = (fwd << 2) | fcode(c);
    }
    if (lastN == -1) {
        const bool f = fwd < rc;
        const uint64_t v = f ? fwd : rc;
        const uint32_t b = (uint32_t)(v >> sh);
        if (!ENUM || (b >= lo && b < hi)) {
            mn = v;
            if (ENUM) {
                const uint32_t pa = 7u, na = a5_of(s[k]);
                mps = f ? pa : a5_cmpl(pa);
                mns = f ? na : a5_cmpl(na);
            }
        }
    }
    int next_win = win;
    for (int i = 1; i <= last; i++) {
        const uint32_t c = s[i + k - 1];
        rc = (rc >> 2) | ((uint64_t)(3u - fcode(c)) << (2 * (k - 1)));
        fwd = ((fwd << 2) | fcode(c)) & mask;
        if (c == 'N') lastN = i + k - 1;
        if (!(i > lastN)) continue;
        const bool f = fwd < rc;
        const uint64_t v = f ? fwd : rc;
        const uint32_t b = (uint32_t)(v >> sh);
        if (ENUM && !(b >= lo && b < hi)) continue;
        uint32_t pa = 0, na = 0;
        if (ENUM) {
            pa = a5_of(s[i - 1]);
            na = (i == last) ? 7u : a5_of(s[i + k]);
            if (!f) { pa = a5_cmpl(pa); na = a5_cmpl(na); }
        }
        if (i > next_win) {
            if (mn != 0) emit(mn, f ? ((mps << 3) | (mns & 7)) : ((mns << 3) | (mps & 7)));
            mn = v; mps = pa; mns = na;
            next_win += win;
            if (next_win + win > last) next_win = last;
        } else if (v < mn || mn == 0) {
            mn = v; mps = pa; mns = na;
        }
    }
    if (mn != 0) emit(mn, (mns << 3) | (mps & 7));
}

__global__ void k_count_min3(const uint8_t *fq, const uint64_t *seq_off, const uint32_t *seq_len, uint64_t r0, uint64_t r1,
                             int k, const uint64_t *chunk_rec, int nchunks, uint32_t *cc, unsigned long long *glob,
                             uint32_t *err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const int sh = 2 * (k - 10);
    for (uint64_t r = r0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < r1; r += stride) {
        const uint32_t L = seq_len[r];
        if (L > (uint32_t)MAX_READ_COUNT) { atomicOr(err, DERR_LONG_READ); continue; }
        uint32_t *ccc = cc ? cc + (size_t)chunk_of(chunk_rec, nchunks, r) * NB : nullptr;
        min3_read<false>(fq + seq_off[r], (int)L, k, 0, 0, [&](uint64_t v, uint32_t) {
            const uint32_t b = (uint32_t)(v >> sh);
            if (ccc) atomicAdd(&ccc[b], 1u); else atomicAdd(&glob[b], 1ull);
        });
    }
}

// Global histogram from per-chunk counts: hist_cnt[b] = sum over chunks.
__global__ void k_sum_chunks(const uint32_t *cc, int nchunks, unsigned long long *glob)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= NB) return;
    unsigned long long s = 0;
    for (int c = 0; c < nchunks; c++) s += cc[(size_t)c * NB + b];
    glob[b] = s;
}

// ------------------------------------------------------------ K2 plain

// The 2-bit packed copy of a piece of the reads (reads r0 .. r0 + n - 1): round offsets off (n + 1, from 0),
// code words w and N masks nm.
struct PackedPiece {
    const uint64_t *off = nullptr, *w = nullptr;
    const uint32_t *nm = nullptr;
    uint64_t r0 = 0;
};

// PK: the bases come from a packed piece (read r of the loop is read pk.r0 + r; seq_len, label, out_off and
// cnt are indexed by that global id), else from the FASTQ bytes.
template <bool WRITE, bool PK = false>
__global__ void __launch_bounds__(256) k_enum_plain(const uint8_t *fq, const uint64_t *seq_off, const uint32_t *seq_len,
                                                    uint64_t n_reads, int k, uint32_t lo, uint32_t hi,
                                                    const uint32_t *label, const uint64_t *out_off, uint32_t *cnt,
                                                    uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id, uint32_t *err,
                                                    PackedPiece pk = PackedPiece{})
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int sh = 2 * (k - 10);
    for (uint64_t lr = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; lr < n_reads; lr += nw) {
        const uint64_t r = PK ? pk.r0 + lr : lr;
        const uint32_t L = seq_len[r];
        if (L <= (uint32_t)k) {
            if (!WRITE && lane == 0) cnt[r] = 0;
            continue;
        }
        if (L > 32u * MAX_ROUNDS_ENUM || L - (uint32_t)k >= 300u) {
            if (lane == 0) { atomicOr(err, DERR_LONG_READ); if (!WRITE) cnt[r] = 0; }
            continue;
        }
        const uint8_t *s = PK ? nullptr : fq + seq_off[r];
        const uint64_t *pw = PK ? pk.w + pk.off[lr] : nullptr;
        const uint32_t *pn = PK ? pk.nm + pk.off[lr] : nullptr;
        const uint32_t nrounds = PK ? (uint32_t)(pk.off[lr + 1] - pk.off[lr]) : 0u;
        auto load = [&](int t, Round &x) {
            if constexpr (PK) load_round_packed(pw, pn, nrounds, t, lane, x);
            else load_round(s, L, t, lane, x);
        };
        const int last = (int)L - k;
        uint64_t base = WRITE ? out_off[r] : 0;
        uint32_t id = (uint32_t)r;
        if (WRITE && label) {
            const uint32_t p = label[r];
            id = (p == BAD) ? (uint32_t)r : p;  // findRoot after full compression (metapart.c:543-568)
        }
        Round prv, cur, nxt;
        load(0, cur);
        load(1, nxt);
        prv = cur;
        uint32_t total = 0;
        for (int t = 0; 32 * t <= last; t++) {
            const int i = 32 * t + lane;
            uint64_t fwd;
            const bool v0 = kmer_at(lane, k, cur, nxt, fwd) && i <= last;
            const uint64_t rc = revcomp(fwd, k);
            const bool f = fwd < rc;
            const uint64_t canon = f ? fwd : rc;
            const uint32_t b = (uint32_t)(canon >> sh);
            const bool v = v0 && b >= lo && b < hi;
            const uint32_t bal = __ballot_sync(FULL, v);
            uint32_t pc = 0, nc = 0;  // characters before and after this lane's k-mer
            if (WRITE) {
                const uint32_t x = __shfl_sync(FULL, cur.c, (lane + 31) & 31), y = __shfl_sync(FULL, prv.c, 31);
                pc = lane ? x : y;
                const int q = lane + k;
                const uint32_t u = __shfl_sync(FULL, cur.c, q & 31), w = __shfl_sync(FULL, nxt.c, q & 31);
                nc = q < 32 ? u : w;
            }
            if (WRITE && v) {
                // 'N' at the read ends (enumerateKmers.c:177, 252-255)
                const uint32_t pa = i > 0 ? a5_of(pc) : 7u, na = i < last ? a5_of(nc) : 7u;
                const uint32_t adj = f ? adj_fwd(pa, na) : adj_rc(pa, na);
                const uint64_t pos = base + __popc(bal & ((1u << lane) - 1));
                o_lo[pos] = (canon << 8) | adj;
                if (o_hi) o_hi[pos] = (uint8_t)(canon >> 56);
                o_id[pos] = id;
            }
            base += __popc(bal);
            total += __popc(bal);
            prv = cur;
            cur = nxt;
            load(t + 2, nxt);
        }
        if (!WRITE && lane == 0) {
            cnt[r] = total;
            if (total > 255) atomicOr(err, DERR_TOO_MANY);  // the reference's per-read counter is a uint8_t
        }
    }
}

// Tuples per read of every scan in one pass: scan s holds buckets [bounds[s], bounds[s+1]).
// cnt[s * stride + r]; S <= MAX_SCAN_COUNT.
constexpr int MAX_SCAN_COUNT = 8;

template <bool PK = false>
__global__ void __launch_bounds__(256) k_enum_count_scans(const uint8_t *fq, const uint64_t *seq_off,
                                                          const uint32_t *seq_len, uint64_t n_reads, int k,
                                                          const uint32_t *bounds, int S, uint32_t *cnt, uint64_t stride,
                                                          uint32_t *err, PackedPiece pk = PackedPiece{})
{
    __shared__ uint32_t sb[MAX_SCAN_COUNT + 1];
    if (threadIdx.x <= (unsigned)S) sb[threadIdx.x] = bounds[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int sh = 2 * (k - 10);
    const uint32_t b_lo = sb[0], b_hi = sb[S];
    for (uint64_t lr = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; lr < n_reads; lr += nw) {
        const uint64_t r = PK ? pk.r0 + lr : lr;
        const uint32_t L = seq_len[r];
        uint32_t c[MAX_SCAN_COUNT];
#pragma unroll
        for (int q = 0; q < MAX_SCAN_COUNT; q++) c[q] = 0;
        if (L > (uint32_t)k && (L > 32u * MAX_ROUNDS_ENUM || L - (uint32_t)k >= 300u)) {
            if (lane == 0) atomicOr(err, DERR_LONG_READ);
        } else if (L > (uint32_t)k) {
            const uint8_t *s = PK ? nullptr : fq + seq_off[r];
            const uint64_t *pw = PK ? pk.w + pk.off[lr] : nullptr;
            const uint32_t *pn = PK ? pk.nm + pk.off[lr] : nullptr;
            const uint32_t nrounds = PK ? (uint32_t)(pk.off[lr + 1] - pk.off[lr]) : 0u;
            auto load = [&](int t, Round &x) {
                if constexpr (PK) load_round_packed(pw, pn, nrounds, t, lane, x);
                else load_round(s, L, t, lane, x);
            };
            const int last = (int)L - k;
            Round cur, nxt;
            load(0, cur);
            load(1, nxt);
            for (int t = 0; 32 * t <= last; t++) {
                const int i = 32 * t + lane;
                uint64_t fwd;
                const bool v0 = kmer_at(lane, k, cur, nxt, fwd) && i <= last;
                const uint64_t rc = revcomp(fwd, k);
                const uint32_t b = (uint32_t)((fwd < rc ? fwd : rc) >> sh);
                if (v0 && b >= b_lo && b < b_hi) {
                    int sc = 0;
#pragma unroll
                    for (int q = 1; q < MAX_SCAN_COUNT; q++) sc += (q < S && b >= sb[q]) ? 1 : 0;
#pragma unroll
                    for (int q = 0; q < MAX_SCAN_COUNT; q++) c[q] += (sc == q) ? 1u : 0u;
                }
                cur = nxt;
                load(t + 2, nxt);
            }
        }
        for (int q = 0; q < S; q++) {
            uint32_t x = c[q];
#pragma unroll
            for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
            if (lane == 0) {
                cnt[(uint64_t)q * stride + r] = x;
                if (x > 255) atomicOr(err, DERR_TOO_MANY);  // the reference's per-read counter is a uint8_t
            }
        }
    }
}

// K2a from the k-mer cache: tuples per read of every scan (S <= MAX_SCAN_COUNT), one warp per read.
// A lane holds at most KC_PER_LANE (< 16) positions of a read, so its counts of the S scans pack into
// 4-bit fields of one word; each scan's count is then one warp reduction.
static_assert(4 * MAX_SCAN_COUNT <= 32 && KC_PER_LANE < 16, "per-lane scan counts are packed in 4-bit fields");
__global__ void __launch_bounds__(256) k_kc_count_scans(const uint64_t *kc_off, const uint64_t *kc_lo,
                                                        const uint8_t *kc_hi, uint64_t n_reads, int k,
                                                        const uint32_t *bounds, int S, uint32_t *cnt, uint64_t stride,
                                                        uint32_t *err)
{
    uint32_t sb[MAX_SCAN_COUNT + 1];  // scan bounds in registers (S + 1 used)
#pragma unroll
    for (int q = 0; q <= MAX_SCAN_COUNT; q++) sb[q] = q <= S ? bounds[q] : 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int sh = 2 * (k - 10);
    const uint32_t b_lo = sb[0], b_hi = sb[S];
    uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint64_t n0 = r < n_reads ? kc_off[r] : 0, n1 = r < n_reads ? kc_off[r + 1] : 0;  // the read's offsets, a read ahead
    for (; r < n_reads; r += nw) {
        const uint64_t p0 = n0, np = n1 - n0;
        if (r + nw < n_reads) {
            n0 = kc_off[r + nw];
            n1 = kc_off[r + nw + 1];
        }
        uint32_t packed = 0;
        if (np > 300) {  // L - k >= 300 (enumerateKmers.c:155)
            if (lane == 0) atomicOr(err, DERR_LONG_READ);
        } else {
            // every position of the read (at most 300: 10 per lane) loaded at once
            uint64_t lv[KC_PER_LANE];
            uint32_t hv[KC_PER_LANE];
#pragma unroll
            for (int t = 0; t < KC_PER_LANE; t++) {
                const uint64_t i = (uint64_t)t * 32 + lane;
                lv[t] = i < np ? kc_lo[p0 + i] : 0ull;
                hv[t] = i < np ? (uint32_t)kc_hi[p0 + i] : (uint32_t)KC_NONE;
            }
#pragma unroll
            for (int t = 0; t < KC_PER_LANE; t++) {
                if ((uint64_t)t * 32 >= np) break;  // uniform across the warp
                const uint64_t km = (lv[t] >> 8) | ((uint64_t)hv[t] << 56);
                const uint32_t b = (uint32_t)(km >> sh);
                if (hv[t] == KC_NONE || b < b_lo || b >= b_hi) continue;
                uint32_t sc = 0;  // scans whose start is at or below b, past the first
#pragma unroll
                for (int q = 1; q < MAX_SCAN_COUNT; q++) sc += b >= sb[q] ? 1u : 0u;
                packed += 1u << (4 * sc);
            }
        }
        for (int q = 0; q < S; q++) {
            const uint32_t x = __reduce_add_sync(FULL, (packed >> (4 * q)) & 15u);
            if (lane == 0) {
                cnt[(uint64_t)q * stride + r] = x;
                if (x > 255) atomicOr(err, DERR_TOO_MANY);  // the reference's per-read counter is a uint8_t
            }
        }
    }
}

// K2b from the k-mer cache: the tuples of buckets [lo, hi) at off[read], in position order.  The
// cache may be one of several pieces: its reads are r0 .. r0 + n_reads - 1 (kc_off is the piece's).
__global__ void __launch_bounds__(256) k_kc_write(const uint64_t *kc_off, const uint64_t *kc_lo, const uint8_t *kc_hi,
                                                  uint64_t r0, uint64_t n_reads, int k, uint32_t lo, uint32_t hi,
                                                  const uint32_t *label, const uint64_t *out_off, uint64_t *o_lo,
                                                  uint8_t *o_hi, uint32_t *o_id)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int sh = 2 * (k - 10);
    uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // the read's offsets, label and output offset, loaded a read ahead
    uint64_t n0 = 0, n1 = 0, nb = 0;
    uint32_t nl = 0;
    if (r < n_reads) {
        n0 = kc_off[r];
        n1 = kc_off[r + 1];
        nb = out_off[r0 + r];
        nl = label ? label[r0 + r] : 0u;
    }
    for (; r < n_reads; r += nw) {
        const uint64_t p0 = n0, np = n1 - n0;
        const uint64_t gr = r0 + r;
        uint64_t base = nb;
        const uint32_t lab = nl;
        if (r + nw < n_reads) {
            n0 = kc_off[r + nw];
            n1 = kc_off[r + nw + 1];
            nb = out_off[gr + nw];
            if (label) nl = label[gr + nw];
        }
        if (np == 0 || np > 300) continue;
        uint32_t id = (uint32_t)gr;
        if (label) id = (lab == BAD) ? (uint32_t)gr : lab;  // findRoot after full compression (metapart.c:543-568)
        // every position of the read (at most 300: 10 per lane) loaded at once
        uint64_t lv[KC_PER_LANE];
        uint32_t hv[KC_PER_LANE];
#pragma unroll
        for (int t = 0; t < KC_PER_LANE; t++) {
            const uint64_t i = (uint64_t)t * 32 + lane;
            lv[t] = i < np ? kc_lo[p0 + i] : 0ull;
            hv[t] = i < np ? (uint32_t)kc_hi[p0 + i] : (uint32_t)KC_NONE;
        }
#pragma unroll
        for (int t = 0; t < KC_PER_LANE; t++) {
            if ((uint64_t)t * 32 >= np) break;  // uniform across the warp
            const uint64_t km = (lv[t] >> 8) | ((uint64_t)hv[t] << 56);
            const uint32_t b = (uint32_t)(km >> sh);
            const bool v = hv[t] != KC_NONE && b >= lo && b < hi;
            const uint32_t bal = __ballot_sync(FULL, v);
            if (v) {
                const uint64_t pos = base + __popc(bal & ((1u << lane) - 1));
                o_lo[pos] = lv[t];
                if (o_hi) o_hi[pos] = (uint8_t)hv[t];
                o_id[pos] = id;
            }
            base += __popc(bal);
        }
    }
}

// ------------------------------------------------------------- K2 3-min

template <bool WRITE>
__global__ void k_enum_min3(const uint8_t *fq, const uint64_t *seq_off, const uint32_t *seq_len, uint64_t n_reads, int k,
                            uint32_t lo, uint32_t hi, const uint32_t *label, const uint64_t *out_off, uint32_t *cnt,
                            uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id, uint32_t *err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += stride) {
        const uint32_t L = seq_len[r];
        if (L > (uint32_t)k && L - (uint32_t)k >= 300u) {
            atomicOr(err, DERR_LONG_READ);
            if (!WRITE) cnt[r] = 0;
            continue;
        }
        uint32_t id = (uint32_t)r;
        if (WRITE && label) { const uint32_t p = label[r]; id = (p == BAD) ? (uint32_t)r : p; }
        uint64_t pos = WRITE ? out_off[r] : 0;
        const uint64_t end = WRITE ? out_off[r + 1] : 0;
        uint32_t c = 0;
        min3_read<true>(fq + seq_off[r], (int)L, k, lo, hi, [&](uint64_t v, uint32_t adj) {
            if constexpr (WRITE) {
                if (pos < end) {
                    o_lo[pos] = (v << 8) | adj;
                    if (o_hi) o_hi[pos] = (uint8_t)(v >> 56);
                    o_id[pos] = id;
                } else {
                    atomicOr(err, DERR_OVERFLOW);
                }
                pos++;
            }
            c++;
        });
        if (!WRITE) {
            cnt[r] = c;
            if (c > 255) atomicOr(err, DERR_TOO_MANY);
        }
    }
}

// ------------------------------------------------------------- host side

// Blocks for `work` items at per_block each, at most `waves` blocks per SM.
static unsigned grid_for(uint64_t work, int per_block, int waves = 16)
{
    const uint64_t max_blocks = (uint64_t)waves * (uint64_t)sm_count();
    uint64_t g = (work + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (unsigned)g;
}

void launch_count(const uint8_t *fq, const ParsedReads &pr, int k, int min3, const uint64_t *chunk_rec, int nchunks,
                  uint32_t *cc, unsigned long long *glob, uint32_t *err, cudaStream_t st, const uint64_t *kc_off,
                  uint64_t *kc_lo, uint8_t *kc_hi, const uint64_t *pk_off, uint64_t *pk_w, uint32_t *pk_n)
{
    if (min3)
        (mp::count_launch(), k_count_min3<<<grid_for(pr.n_reads, 128, 32), 128, 0, st>>>(fq, pr.seq_off, pr.seq_len, 0, pr.n_reads, k,
                                                                          chunk_rec, nchunks, cc, glob, err));
    else
        (mp::count_launch(), (pk_w ? k_count_plain<true> : k_count_plain<false>)<<<grid_for(pr.n_reads, 8), 256, 0, st>>>(
            fq, pr.seq_off, pr.seq_len, 0, pr.n_reads, k, chunk_rec, nchunks, cc, glob, err, kc_off, kc_lo, kc_hi, pk_off,
            pk_w, pk_n));
    if (cc && glob) (mp::count_launch(), k_sum_chunks<<<NB / 256, 256, 0, st>>>(cc, nchunks, glob));
}

void launch_enum_count(const uint8_t *fq, const ParsedReads &pr, int k, int min3, uint32_t lo, uint32_t hi,
                       uint32_t *cnt, uint32_t *err, cudaStream_t st)
{
    if (min3)
        (mp::count_launch(), k_enum_min3<false><<<grid_for(pr.n_reads, 128, 32), 128, 0, st>>>(
            fq, pr.seq_off, pr.seq_len, pr.n_reads, k, lo, hi, nullptr, nullptr, cnt, nullptr, nullptr, nullptr, err));
    else
        (mp::count_launch(), k_enum_plain<false><<<grid_for(pr.n_reads, 8), 256, 0, st>>>(fq, pr.seq_off, pr.seq_len, pr.n_reads, k, lo, hi,
                                                                     nullptr, nullptr, cnt, nullptr, nullptr, nullptr, err));
}

int launch_enum_count_scans(const uint8_t *fq, const ParsedReads &pr, int k, const uint32_t *bounds, int S,
                            uint32_t *cnt, uint64_t stride, uint32_t *err, cudaStream_t st)
{
    if (S < 1 || S > MAX_SCAN_COUNT) return -1;
    (mp::count_launch(), k_enum_count_scans<<<grid_for(pr.n_reads, 8), 256, 0, st>>>(
        fq, pr.seq_off, pr.seq_len, pr.n_reads, k, bounds, S, cnt, stride, err));
    return 0;
}

void launch_pk_rounds(const ParsedReads &pr, int k, uint32_t *nr, cudaStream_t st)
{
    (mp::count_launch(), k_pk_rounds<<<(unsigned)((pr.n_reads + 255) / 256), 256, 0, st>>>(pr.seq_len, pr.n_reads, k, nr));
}

static PackedPiece packed_piece(const uint64_t *off, const uint64_t *w, const uint32_t *nm, uint64_t r0)
{
    PackedPiece p;
    p.off = off;
    p.w = w;
    p.nm = nm;
    p.r0 = r0;
    return p;
}

int launch_pk_count_scans(const uint64_t *pk_off, const uint64_t *pk_w, const uint32_t *pk_n, uint64_t r0, uint64_t n_reads,
                          const uint32_t *seq_len, int k, const uint32_t *bounds, int S, uint32_t *cnt, uint64_t stride,
                          uint32_t *err, cudaStream_t st)
{
    if (S < 1 || S > MAX_SCAN_COUNT) return -1;
    if (n_reads == 0) return 0;
    (mp::count_launch(), k_enum_count_scans<true><<<grid_for(n_reads, 8), 256, 0, st>>>(
        nullptr, nullptr, seq_len, n_reads, k, bounds, S, cnt, stride, err, packed_piece(pk_off, pk_w, pk_n, r0)));
    return 0;
}

void launch_pk_count(const uint64_t *pk_off, const uint64_t *pk_w, const uint32_t *pk_n, uint64_t r0, uint64_t n_reads,
                     const uint32_t *seq_len, int k, uint32_t lo, uint32_t hi, uint32_t *cnt, uint32_t *err, cudaStream_t st)
{
    if (n_reads == 0) return;
    (mp::count_launch(), k_enum_plain<false, true><<<grid_for(n_reads, 8), 256, 0, st>>>(
        nullptr, nullptr, seq_len, n_reads, k, lo, hi, nullptr, nullptr, cnt, nullptr, nullptr, nullptr, err,
        packed_piece(pk_off, pk_w, pk_n, r0)));
}

void launch_pk_write(const uint64_t *pk_off, const uint64_t *pk_w, const uint32_t *pk_n, uint64_t r0, uint64_t n_reads,
                     const uint32_t *seq_len, int k, uint32_t lo, uint32_t hi, const uint32_t *label, const uint64_t *off,
                     uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id, uint32_t *err, cudaStream_t st)
{
    if (n_reads == 0) return;
    (mp::count_launch(), k_enum_plain<true, true><<<grid_for(n_reads, 8), 256, 0, st>>>(
        nullptr, nullptr, seq_len, n_reads, k, lo, hi, label, off, nullptr, o_lo, o_hi, o_id, err,
        packed_piece(pk_off, pk_w, pk_n, r0)));
}

void launch_kc_positions(const ParsedReads &pr, int k, uint32_t *npos, cudaStream_t st)
{
    (mp::count_launch(), k_kc_positions<<<(unsigned)((pr.n_reads + 255) / 256), 256, 0, st>>>(pr.seq_len, pr.n_reads, k, npos));
}

int launch_kc_count_scans(const uint64_t *kc_off, const uint64_t *kc_lo, const uint8_t *kc_hi, uint64_t n_reads, int k,
                          const uint32_t *bounds, int S, uint32_t *cnt, uint64_t stride, uint32_t *err, cudaStream_t st)
{
    if (S < 1 || S > MAX_SCAN_COUNT) return -1;
    (mp::count_launch(), k_kc_count_scans<<<grid_for(n_reads, 8), 256, 0, st>>>(kc_off, kc_lo, kc_hi, n_reads, k, bounds, S,
                                                                             cnt, stride, err));
    return 0;
}

void launch_kc_write(const uint64_t *kc_off, const uint64_t *kc_lo, const uint8_t *kc_hi, uint64_t r0, uint64_t n_reads,
                     int k, uint32_t lo, uint32_t hi, const uint32_t *label, const uint64_t *off, uint64_t *o_lo,
                     uint8_t *o_hi, uint32_t *o_id, cudaStream_t st)
{
    if (n_reads == 0) return;
    (mp::count_launch(), k_kc_write<<<grid_for(n_reads, 8), 256, 0, st>>>(kc_off, kc_lo, kc_hi, r0, n_reads, k, lo, hi,
                                                                       label, off, o_lo, o_hi, o_id));
}

void launch_enum_write(const uint8_t *fq, const ParsedReads &pr, int k, int min3, uint32_t lo, uint32_t hi,
                       const uint32_t *label, const uint64_t *off, uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id,
                       uint32_t *err, cudaStream_t st)
{
    if (min3)
        (mp::count_launch(), k_enum_min3<true><<<grid_for(pr.n_reads, 128, 32), 128, 0, st>>>(
            fq, pr.seq_off, pr.seq_len, pr.n_reads, k, lo, hi, label, off, nullptr, o_lo, o_hi, o_id, err));
    else
        (mp::count_launch(), k_enum_plain<true><<<grid_for(pr.n_reads, 8), 256, 0, st>>>(fq, pr.seq_off, pr.seq_len, pr.n_reads, k, lo, hi,
                                                                    label, off, nullptr, o_lo, o_hi, o_id, err));
}

}  // namespace mp
