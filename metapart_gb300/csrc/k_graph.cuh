#pragma once
#include <vector>

#include "k_reads.cuh"

namespace mp {

// Sorted tuples of one scan (views into the sort buffers) plus the filter's zero marks.
struct Tuples {
    uint64_t *lo = nullptr;   // kmer << 8 | adj
    uint8_t *hi = nullptr;    // kmer >> 56 (nullable)
    uint32_t *id = nullptr;   // read id / component label
    uint64_t n = 0;
    uint32_t *z = nullptr;    // zero marks of the filter, one bit per tuple
};

// K4: markMischiefKmers over the scan; range_bounds = T + 1 tuple bounds of the thread ranges.
// multi: the ranges of several scans one after another (a batch of samples), whose boundaries may cut a run.
int filter_scan(Tuples &tp, const std::vector<uint64_t> &range_bounds, uint32_t *parent, uint8_t *filtered,
                DeviceArena &arena, cudaStream_t st, bool apply_zero, bool multi = false);
// K5: unionFindPar2 + unionFind + printStats compression for the scan.  rebad: a read flagged in an
// earlier scan whose parent is not BAD (the first read an earlier scan hooked below a component), marked
// BAD again first; ~0u for none.  *hooked: the scan's BAD first read when it was hooked below the
// component of the scan's last run (~0u otherwise), for the next scan's rebad.
int union_scan(Tuples &tp, const std::vector<uint64_t> &range_bounds, uint32_t *parent, const uint8_t *filtered,
               uint64_t n_reads, DeviceArena &arena, cudaStream_t st, uint32_t rebad, uint32_t *hooked);
// K5 for one piece of a scan split by bucket ranges (the scan's tuples do not fit at once): the sweep of
// unionFindPar2 over the piece's part of the thread ranges.  bounds: T' + 1 tuple bounds of those parts;
// seen[t] = 1 when part t's thread range had a valid tuple in an earlier piece; init_*: the scan's initial
// sweep state (its last tuple's k-mer after the filter, its first tuple's read, whether that read was BAD
// when the scan's unions began).  On return has_valid[t] = 1 when part t holds a valid tuple.  No
// compression (compress_parents, once the scan's last piece is done).  With a BAD first read, *anchor_v
// (device) receives the read of the range's first valid tuple when that tuple carries init_kmer; after
// the last piece, hook_bad_anchor does what union_scan does with it.
int union_piece(Tuples &tp, const std::vector<uint64_t> &bounds, const std::vector<uint8_t> &seen, uint64_t init_kmer,
                uint32_t init_min, bool init_min_ok, uint32_t *parent, const uint8_t *filtered, DeviceArena &arena,
                cudaStream_t st, std::vector<uint8_t> &has_valid, uint32_t *anchor_v);
void rebad_read(uint32_t *parent, uint32_t r, cudaStream_t st);
// Reads whose parent is neither BAD nor a root, counted on st into *out (d_count: one device word).
int count_nonroot(const uint32_t *parent, uint64_t n, unsigned long long *d_count, cudaStream_t st, uint64_t *out);
void hook_bad_anchor(uint32_t *parent, uint32_t b, const uint32_t *anchor_v, uint32_t *hooked, cudaStream_t st);
void compress_parents(uint32_t *parent, uint64_t n_reads, cudaStream_t st);
// K6: sizes, unionFindPeReads(1000), final compression and the 17 partition bounds (host).
int mate_union_and_plan(uint32_t *parent, uint64_t n_reads, uint32_t *size, uint64_t *bounds_out, DeviceArena &arena,
                        cudaStream_t st, int *rounds_out);
// The same without the partition bounds (sizes recounted after the final compression).
int mate_union(uint32_t *parent, uint64_t n_reads, uint32_t *size, DeviceArena &arena, cudaStream_t st, int *rounds_out);
int plan_partitions(const uint32_t *parent, const uint32_t *size, uint64_t n_reads, uint64_t *bounds_host,
                    DeviceArena &arena, cudaStream_t st);

// Batches of samples, one after another in the tuple array and the read ids (every sample one scan).
// K5 for all of them: range_bounds = R + 1 tuple bounds of every sample's thread ranges in order,
// range_seg[t] = the sample of range t, seg_tstart = nseg + 1 tuple offsets of the samples.
int union_segments(Tuples &tp, const std::vector<uint64_t> &range_bounds, const std::vector<uint32_t> &range_seg,
                   const std::vector<uint64_t> &seg_tstart, uint32_t *parent, const uint8_t *filtered, uint64_t n_reads,
                   DeviceArena &arena, cudaStream_t st);
// The 16 work partitions of every sample (seg_reads: nseg + 1 read offsets); bounds_host: nseg x 17, in
// each sample's own read ids.
int plan_partitions_segments(const uint32_t *parent, const uint32_t *size, uint64_t n_reads,
                             const std::vector<uint64_t> &seg_reads, uint64_t *bounds_host, DeviceArena &arena,
                             cudaStream_t st);

}  // namespace mp
