#pragma once
#include <vector>

#include "k_reads.cuh"

namespace mp {

// Where every record goes in the concatenated partition files (file j = partition * T + tid): the
// entries' units in file order (val), their byte offsets (off), the total; persistent arena arrays.
struct OutputPlan {
    uint32_t *val = nullptr;
    uint64_t *off = nullptr;
    uint64_t n = 0, total = 0;
    const uint64_t *rec_start = nullptr;
    int interleaved = 0;
};

// The plan; file_sizes: 16 * T byte counts in file order.
int plan_output(const uint8_t *d_fq, const ParsedReads &pr, const uint32_t *d_label, const uint64_t *bounds_host,
                const uint64_t *chunk_rec_host, int nchunks, int T, int interleaved, OutputPlan *plan,
                std::vector<uint64_t> &file_sizes, DeviceArena &arena, cudaStream_t st);

// The same for a batch of samples one after another in the read ids (seg_reads: nseg + 1 read offsets;
// d_label: global root ids; bounds_host: nseg x 17 in each sample's ids; chunk_rec_host[q]: sample q's
// nchunks + 1 chunk record starts in its own ids; T[q] its numThreads).  Sample q's files are the global
// files file0[q] .. file0[q + 1] - 1 (file0: nseg + 1 entries, filled here), laid out one after another.
int plan_output_batch(const ParsedReads &pr, const uint32_t *d_label, int interleaved, const std::vector<uint64_t> &seg_reads,
                      const std::vector<uint64_t> &bounds_host, const std::vector<std::vector<uint64_t>> &chunk_rec_host,
                      const std::vector<int> &T, OutputPlan *plan, std::vector<uint64_t> &file_sizes,
                      std::vector<uint64_t> &file0, DeviceArena &arena, cudaStream_t st);

// The records' bytes to dst (plan.total bytes, 4-byte aligned device memory); _range: the entries
// [e0, e1) only (their bytes [off[e0], off[e1]) of dst).
int copy_output(const OutputPlan &plan, const uint8_t *d_fq, uint8_t *dst, cudaStream_t st);
int copy_output_range(const OutputPlan &plan, uint64_t e0, uint64_t e1, const uint8_t *d_fq, uint8_t *dst,
                      cudaStream_t st);

}  // namespace mp
