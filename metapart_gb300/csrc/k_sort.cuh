#pragma once
#include <vector>

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
    double seg_ms = 0;        // shared-memory unit sort (bucket_sort)
    double big_ms = 0;        // oversized buckets (bucket_sort)
    uint64_t units = 0, big_buckets = 0, big_tuples = 0;
    uint64_t unit_passes = 0;                 // unit sort: digit passes, summed over units
    uint64_t phase_cycles[3] = {0, 0, 0};     // unit sort: SM cycles summed over units in load, passes, store
    uint64_t pass_cycles[7] = {};  // bucket digit passes: SM cycles summed over tiles in the tile-id fetch, loads +
                                   //   ranks, digit scan, tile order + look-back, stores; then digit 0's look-back
                                   //   status words read and polls of unposted words, summed over tiles
};

// Adjacent tuple pairs of lo/hi (hi nullable) out of (k-mer, adjacency) order, counted on st into *out
// (d_count: one device word of scratch).
int count_unsorted(const uint64_t *lo, const uint8_t *hi, uint64_t n, unsigned long long *d_count, cudaStream_t st,
                   uint64_t *out);

// Stable sort of b[cur][0, n) by (hi, lo); on return b.cur names the sorted buffer.
int radix_sort(SortBufs &b, uint64_t n, bool has_hi, DeviceArena &arena, cudaStream_t st, SortStats *stats);

// Independent tuple sets (samples) one after another in one tuple array: segment q holds the tuples
// [tstart[q], tstart[q + 1]) and the m-mer buckets q * NB .. q * NB + NB - 1 of a segmented histogram.
struct SortSegments {
    int nseg = 0;
    std::vector<uint64_t> tstart;  // nseg + 1 tuple offsets (host)
};

// Stable sort of one scan's tuples by (k-mer, adjacency) using the scan's m-mer bucket counts
// (d_hist: the 1048577-entry .kmerHist prefix in device memory, buckets [scan_lo, scan_hi)).  On return
// lo/id are in b.*[*out_lo_buf] and hi in b.hi[*out_hi_buf].  With segs, each segment is sorted on its own
// (its tuples stay in its range): d_hist is then the prefix over the segments' buckets one after another
// (nseg * NB + 1 entries, tuple offsets into the whole array) and [scan_lo, scan_hi) = [0, nseg * NB).
int bucket_sort(SortBufs &b, uint64_t n, bool has_hi, int k, const uint64_t *d_hist, uint64_t scan_lo, uint64_t scan_hi,
                DeviceArena &arena, cudaStream_t st, SortStats *stats, int *out_lo_buf, int *out_hi_buf,
                const SortSegments *segs = nullptr);

}  // namespace mp
