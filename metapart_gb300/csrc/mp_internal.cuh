// Host-side pieces shared by the job driver (mp_api.cu) and the batch driver (mp_batch.cu).
#pragma once
#include "k_reads.cuh"

namespace mp {

// A piece of the k-mer cache: the reads r0 .. r0 + n - 1, their position offsets off (n + 1, from 0)
// and per position lo = canon << 8 | adj, hi = canon >> 56 (KC_NONE: the window holds an N).
struct KcPiece {
    uint64_t r0 = 0, n = 0;
    uint64_t *off = nullptr, *lo = nullptr;
    uint8_t *hi = nullptr;
};

// One cache piece for the reads of pr (global reads r0 ..): position offsets by a scan of L - k + 1,
// and the lo/hi arrays, persistent in arena; false (nothing kept) when device memory or the budget does
// not allow it.
bool make_kc_piece(DeviceArena &arena, cudaStream_t st, const ParsedReads &pr, uint64_t r0, int k, KcPiece *out);
void free_kc_piece(DeviceArena &arena, KcPiece &q);

// The context's device and its HBM budget accounting (shared by every job and batch of the context).
int ctx_device(const mp_ctx *ctx);
void ctx_budget(mp_ctx *ctx, std::atomic<uint64_t> **used, uint64_t *limit);

// parent[x] = x for every read.
void launch_init_parent(uint32_t *parent, uint64_t n, cudaStream_t st);

// Device time of the work queued on a stream while the timer lives, added to *slot (ms).
struct StageTimer {
    cudaEvent_t a, b;
    cudaStream_t st;
    double *acc;
    StageTimer(cudaStream_t s, double *slot) : st(s), acc(slot)
    {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, st);
    }
    ~StageTimer()
    {
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        *acc += ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    StageTimer(const StageTimer &) = delete;
    StageTimer &operator=(const StageTimer &) = delete;
};

}  // namespace mp
