// Shared device/host definitions of the GB300 read-partitioning path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "metapart_gpu.h"

namespace mp {

constexpr uint32_t NB = 1u << 20;            // 4^10 m-mer buckets (m is 10 in the reference)
constexpr uint32_t BAD = 0xFFFFFFFFu;        // parent value of a filtered read (reference: 0xBADBADBAD)
constexpr int WARP = 32;
constexpr int MAX_ROUNDS_ENUM = 11;          // reads up to 352 bases in metapart (reference asserts L-k < 300)
constexpr int MAX_READ_COUNT = 4096;         // longest read accepted by the counting stage

// Device error flags (set by kernels, read by the host after a stage).
enum DevErr : uint32_t {
    DERR_NONE = 0,
    DERR_SPIN = 1u << 0,       // a bounded wait gave up (look-back, union retries)
    DERR_LONG_READ = 1u << 1,  // read longer than the kernel supports
    DERR_OVERFLOW = 1u << 2,   // more output than the count pass reserved
    DERR_TOO_MANY = 1u << 3,   // a read has 256 or more tuples in one scan
    DERR_NONACGT = 1u << 4,    // a sequence byte other than A, C, G, T, N (no packed copy of the reads)
};

// Iteration limits of the device's bounded waits: the sort's look-back polls of one status word, the
// union-find's hook retries, and the mate union's rounds.  A wait that runs out sets DERR_SPIN (or the
// round count ends the stage) and the call returns MP_EDEVICE; nothing waits without a limit.
struct WaitLimits {
    uint32_t lookback_spins = 1u << 22;
    uint32_t union_retries = 1u << 20;
    uint32_t mate_rounds = 4000000u;
};

struct DevStatus {
    uint32_t err;
    uint32_t pad;
    unsigned long long counter;
};

__host__ __device__ inline uint64_t kmer_mask(int k) { return (k >= 32) ? ~0ull : ((1ull << (2 * k)) - 1); }

// Reverse complement of a 2k-bit forward code (A0 C1 G2 T3; complement = 3 - code).
// Equals the reference's rolling curRcInt (countMmers.c:120-137, 175-181).
__device__ __forceinline__ uint64_t revcomp(uint64_t fwd, int k)
{
    uint64_t r = __brevll(fwd);
    r = ((r >> 1) & 0x5555555555555555ull) | ((r & 0x5555555555555555ull) << 1);
    return (r >> (64 - 2 * k)) ^ kmer_mask(k);
}

// Base code of a FASTQ byte: charToIntMap[(c & 6) >> 1] = {0,1,3,2} (countMmers.c:85)
__host__ __device__ __forceinline__ uint32_t fcode(uint32_t c)
{
    uint32_t x = (c >> 1) & 3;
    return x ^ (x >> 1);  // 0->0, 1->1, 2->3, 3->2
}

// Bits 1..5 of a byte: the only bits the adjacency byte uses (enumerateKmers.c:215, 239).
// adj(fwd) = a5(prev) << 3 | (a5(next) & 7);  complement via "TGAC   N"[a5 & 7].
__host__ __device__ __forceinline__ uint32_t a5_of(uint32_t c) { return (c >> 1) & 0x1F; }
__host__ __device__ __forceinline__ uint32_t a5_cmpl(uint32_t a5)
{
    // a5 of "TGAC   N"[a5 & 7]: T=0x0A G=0x03 A=0x00 C=0x01 ' '=0x10 N=0x07
    const uint64_t tab = 0x071010100100030Aull;  // byte j = a5 of table entry j
    return (uint32_t)((tab >> (8 * (a5 & 7))) & 0xFF);
}
__host__ __device__ __forceinline__ uint32_t adj_fwd(uint32_t pa5, uint32_t na5) { return ((pa5 << 3) & 0xF8) | (na5 & 7); }
__host__ __device__ __forceinline__ uint32_t adj_rc(uint32_t pa5, uint32_t na5)
{
    // prev' = cmpl(prev), next' = cmpl(next); adj = ((next' << 2) & 0xF8) | ((prev' >> 1) & 7)
    return ((a5_cmpl(na5) << 3) & 0xF8) | (a5_cmpl(pa5) & 7);
}

// Process-wide count of kernels this library launched (mp_launch_count).
void count_launch();

// Streaming multiprocessors of the current device (grids of persistent and grid-stride kernels are sized
// in multiples of it).
int sm_count();

// Device-wide exclusive scans (k_reads.cu).
void scan_u32_to_u64(const uint32_t *in, uint64_t *out, uint64_t n, uint64_t *total_dev, void *tmp, size_t tmp_bytes,
                     cudaStream_t st);
void scan_u64(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t *total_dev, void *tmp, size_t tmp_bytes,
              cudaStream_t st);
size_t scan_tmp_bytes(uint64_t n);

}  // namespace mp

#define MP_CUDA(x)                                                                                   \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) return mp::set_cuda_error(e_, #x, __FILE__, __LINE__);                \
    } while (0)

namespace mp {
int set_cuda_error(cudaError_t e, const char *what, const char *file, int line);
int set_error(int code, const char *fmt, ...);
}  // namespace mp
