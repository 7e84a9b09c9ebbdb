// Host-side pieces shared by the job driver (mp_api.cu) and the batch driver (mp_batch.cu).
#pragma once
#include <nvtx3/nvToolsExt.h>
#include "k_reads.cuh"

namespace mp {

// A piece of the count pass's copy of the reads for the partition's enumeration, the reads r0 .. r0 + n - 1,
// in one of two forms.  k-mer cache (lo non-null): position offsets off (n + 1, from 0) and per position
// lo = canon << 8 | adj, hi = canon >> 56 (KC_NONE: the window holds an N) -- 9 bytes per position, and
// the enumeration only filters it.  Packed reads (pw non-null): round offsets poff (n + 1, from 0) and per
// round of 32 bases a 2-bit code word pw and an N mask pn -- 0.375 bytes per base, and the enumeration
// recomputes the k-mers.
struct KcPiece {
    uint64_t r0 = 0, n = 0;
    uint64_t *off = nullptr, *lo = nullptr;
    uint8_t *hi = nullptr;
    uint64_t *poff = nullptr, *pw = nullptr;
    uint32_t *pn = nullptr;
};

// One piece for the reads of pr (global reads r0 ..), persistent in arena: the k-mer cache (offsets by a
// scan of L - k + 1) or the packed reads (offsets by a scan of ceil(L / 32)); false (nothing kept) when
// device memory or the budget does not allow it.
bool make_kc_piece(DeviceArena &arena, cudaStream_t st, const ParsedReads &pr, uint64_t r0, int k, KcPiece *out);
bool make_pk_piece(DeviceArena &arena, cudaStream_t st, const ParsedReads &pr, uint64_t r0, int k, KcPiece *out);
void free_kc_piece(DeviceArena &arena, KcPiece &q);

int store_count_scans(const KcPiece &q, const uint32_t *seq_len, int k, const uint32_t *bounds, int S, uint32_t *cnt,
                      uint64_t stride, uint32_t *err, cudaStream_t st);
void store_write(const KcPiece &q, const uint32_t *seq_len, int k, uint32_t lo, uint32_t hi, const uint32_t *label,
                 const uint64_t *off, uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id, uint32_t *err, cudaStream_t st);

// Read stores of a job (mp_job_set_read_store).
constexpr int STORE_FASTQ = MP_STORE_FASTQ, STORE_KMER_CACHE = MP_STORE_KMER_CACHE, STORE_PACKED = MP_STORE_PACKED;

// The context's device and its HBM budget accounting (shared by every job and batch of the context).
int ctx_device(const mp_ctx *ctx);
void ctx_budget(mp_ctx *ctx, std::atomic<uint64_t> **used, uint64_t *limit);

// parent[x] = x for every read.
void launch_init_parent(uint32_t *parent, uint64_t n, cudaStream_t st);

// Device time of the work queued on a stream while the timer lives, added to *slot (ms).
// The stages of a job or batch, in the order of their time slots (mp_job_stage_ms, mp_batch_stage_ms).
constexpr const char *STAGE_NAMES[8] = {"parse", "count", "enumerate", "sort", "filter", "union_find",
                                        "mate_union_plan", "output"};

// A stage's device time (CUDA events on its stream, added to its slot) and an NVTX range of the stage's
// name for a profiler's timeline (a no-op without one attached).
struct StageTimer {
    cudaEvent_t a, b;
    cudaStream_t st;
    double *acc;
    StageTimer(cudaStream_t s, double *slots, int stage) : st(s), acc(slots + stage)
    {
        nvtxRangePushA(STAGE_NAMES[stage]);
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
        nvtxRangePop();
    }
    StageTimer(const StageTimer &) = delete;
    StageTimer &operator=(const StageTimer &) = delete;
};

}  // namespace mp
