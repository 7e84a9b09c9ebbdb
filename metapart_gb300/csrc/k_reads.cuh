// Device memory arena, the parsed-read table and the host-side stage entry points.
#pragma once
#include <atomic>
#include <vector>

#include "mp_common.cuh"

namespace mp {

// Stream-ordered device allocations of one job.  Scratch allocations live until
// release_scratch(); persistent ones until release_all().  Sizes are charged
// against the context's HBM budget, which jobs running on other host threads share.
struct DeviceArena {
    cudaStream_t st = nullptr;
    std::vector<std::pair<void *, size_t>> persistent, scratch;
    std::atomic<uint64_t> *budget_used = nullptr;  // shared with the context
    uint64_t budget_limit = ~0ull;
    uint64_t peak = 0, live = 0;
    WaitLimits lim;  // the bounded waits of the kernels this arena's work launches

    void *raw(size_t bytes, bool keep)
    {
        bytes = (bytes + 255) & ~(size_t)255;
        if (bytes == 0) bytes = 256;
        if (budget_used) {  // reserve first, so concurrent jobs never overshoot the budget together
            uint64_t cur = budget_used->load();
            do {
                if (cur + bytes > budget_limit) return nullptr;
            } while (!budget_used->compare_exchange_weak(cur, cur + bytes));
        }
        void *p = nullptr;
        if (cudaMallocAsync(&p, bytes, st) != cudaSuccess) {
            cudaGetLastError();
            if (budget_used) budget_used->fetch_sub(bytes);
            return nullptr;
        }
        (keep ? persistent : scratch).push_back({p, bytes});
        live += bytes;
        if (live > peak) peak = live;
        return p;
    }
    template <typename T> T *alloc(size_t n) { return (T *)raw(n * sizeof(T), false); }
    template <typename T> T *alloc_persistent(size_t n) { return (T *)raw(n * sizeof(T), true); }
    void free_one(std::vector<std::pair<void *, size_t>> &v, void *p)
    {
        for (size_t i = 0; i < v.size(); i++)
            if (v[i].first == p) {
                cudaFreeAsync(p, st);
                if (budget_used) budget_used->fetch_sub(v[i].second);
                live -= v[i].second;
                v.erase(v.begin() + (long)i);
                return;
            }
    }
    void free_persistent(void *p) { if (p) free_one(persistent, p); }
    void free_scratch(void *p) { if (p) free_one(scratch, p); }
    void release_scratch()
    {
        for (auto &x : scratch) {
            cudaFreeAsync(x.first, st);
            if (budget_used) budget_used->fetch_sub(x.second);
            live -= x.second;
        }
        scratch.clear();
    }
    void release_all()
    {
        release_scratch();
        for (auto &x : persistent) {
            cudaFreeAsync(x.first, st);
            if (budget_used) budget_used->fetch_sub(x.second);
            live -= x.second;
        }
        persistent.clear();
    }
};

// CUDA events owned by a scope: destroyed on every return path.
struct Events {
    std::vector<cudaEvent_t> ev;
    explicit Events(size_t n, unsigned flags = cudaEventDefault) : ev(n, nullptr)
    {
        for (auto &e : ev)
            if (cudaEventCreateWithFlags(&e, flags) != cudaSuccess) e = nullptr;
    }
    ~Events()
    {
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
    Events(const Events &) = delete;
    Events &operator=(const Events &) = delete;
    cudaEvent_t &operator[](size_t i) { return ev[i]; }
    size_t size() const { return ev.size(); }
};

struct ParsedReads {
    uint64_t n_reads = 0;
    uint64_t *rec_start = nullptr;  // n_reads + 1 record start offsets (last = input size)
    uint64_t *seq_off = nullptr;    // sequence line offset of each record
    uint32_t *seq_len = nullptr;    // sequence length of each record
};

int parse_fastq(const uint8_t *d_buf, uint64_t n, ParsedReads *pr, DeviceArena &arena, cudaStream_t st);
// The same for the bytes [begin, end) of a 16-byte aligned buffer (offsets relative to begin).
int parse_fastq_range(const uint8_t *d_base, uint64_t begin, uint64_t end, ParsedReads *pr, DeviceArena &arena,
                      cudaStream_t st);
// Copies a segment's record table (parsed from the segment alone) into dst at read r0, its offsets
// moved by byte_base; dst's arrays hold all reads.
void concat_records(const ParsedReads &seg, uint64_t byte_base, ParsedReads &dst, uint64_t r0, cudaStream_t st);
int records_at_offsets(const ParsedReads *pr, const uint64_t *h_offsets, int nq, uint64_t *h_rec, DeviceArena &arena,
                       cudaStream_t st);

}  // namespace mp
