#pragma once
#include "k_reads.cuh"

namespace mp {

// Ping-pong tuple buffers: lo = kmer << 8 | adj, hi = kmer >> 56 (only when 2k + 8 > 64), id = read id.
struct SortBufs {
    uint64_t *lo[2] = {nullptr, nullptr};
    uint8_t *hi[2] = {nullptr, nullptr};
    uint32_t *id[2] = {nullptr, nullptr};
    int cur = 0;
};

struct SortStats {
    uint64_t tuples = 0;
    int passes = 0;
    double hist_ms = 0;
    double pass_ms = 0;
    uint64_t bytes = 0;       // algorithmic bytes of the digit passes (read + write of every tuple per pass)
    uint64_t hist_bytes = 0;  // bytes read by the upfront histogram
};

// Stable sort of b[cur][0, n) by (hi, lo); on return b.cur names the sorted buffer.
int radix_sort(SortBufs &b, uint64_t n, bool has_hi, DeviceArena &arena, cudaStream_t st, SortStats *stats);

}  // namespace mp
