#pragma once
#include <vector>

#include "k_reads.cuh"

namespace mp {

// Builds the concatenated partition files in device memory (persistent allocation of the arena).
// file_sizes: 16 * T byte counts in file order j = partition * T + tid.
int gather_output(const uint8_t *d_fq, const ParsedReads &pr, const uint32_t *d_label, const uint64_t *bounds_host,
                  const uint64_t *chunk_rec_host, int nchunks, int T, int interleaved, uint8_t **d_out,
                  uint64_t *total_out, std::vector<uint64_t> &file_sizes, DeviceArena &arena, cudaStream_t st);

}  // namespace mp
