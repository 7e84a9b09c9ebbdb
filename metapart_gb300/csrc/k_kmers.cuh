#pragma once
#include "k_reads.cuh"

namespace mp {

// K1: bucket counts.  cc (nullable): per-chunk u32 counts [nchunks][NB]; glob: u64 counts [NB]
// (summed from cc when cc is given; nullable with cc).
// kc_off/kc_lo/kc_hi (nullable, plain variant only): the k-mer cache to fill (see k_kc_*).
// pk_off/pk_w/pk_n (nullable, plain variant only): the 2-bit packed copy of the reads to fill: per read with a
// k-mer, ceil(L / 32) rounds (a code word, most significant base first, and an N mask) at pk_off[read];
// an input byte other than A, C, G, T, N sets DERR_NONACGT in err (the copy is then unusable).
void launch_count(const uint8_t *fq, const ParsedReads &pr, int k, int min3, const uint64_t *chunk_rec, int nchunks,
                  uint32_t *cc, unsigned long long *glob, uint32_t *err, cudaStream_t st, const uint64_t *kc_off = nullptr,
                  uint64_t *kc_lo = nullptr, uint8_t *kc_hi = nullptr, const uint64_t *pk_off = nullptr,
                  uint64_t *pk_w = nullptr, uint32_t *pk_n = nullptr);

// Packed copy: rounds per read; the enumeration of one piece (reads r0 .. r0 + n_reads - 1; seq_len, cnt,
// label and off indexed by global read id): every scan's per-read tuple counts, one range's counts, and
// one range's tuples -- the FASTQ enumeration's results from the packed bases.
void launch_pk_rounds(const ParsedReads &pr, int k, uint32_t *nr, cudaStream_t st);
int launch_pk_count_scans(const uint64_t *pk_off, const uint64_t *pk_w, const uint32_t *pk_n, uint64_t r0, uint64_t n_reads,
                          const uint32_t *seq_len, int k, const uint32_t *bounds, int S, uint32_t *cnt, uint64_t stride,
                          uint32_t *err, cudaStream_t st);
void launch_pk_count(const uint64_t *pk_off, const uint64_t *pk_w, const uint32_t *pk_n, uint64_t r0, uint64_t n_reads,
                     const uint32_t *seq_len, int k, uint32_t lo, uint32_t hi, uint32_t *cnt, uint32_t *err, cudaStream_t st);
void launch_pk_write(const uint64_t *pk_off, const uint64_t *pk_w, const uint32_t *pk_n, uint64_t r0, uint64_t n_reads,
                     const uint32_t *seq_len, int k, uint32_t lo, uint32_t hi, const uint32_t *label, const uint64_t *off,
                     uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id, uint32_t *err, cudaStream_t st);

// k-mer cache: positions per read (L - k + 1 or 0); per-read tuple counts of every scan; one scan's tuples.
void launch_kc_positions(const ParsedReads &pr, int k, uint32_t *npos, cudaStream_t st);
int launch_kc_count_scans(const uint64_t *kc_off, const uint64_t *kc_lo, const uint8_t *kc_hi, uint64_t n_reads, int k,
                          const uint32_t *bounds, int S, uint32_t *cnt, uint64_t stride, uint32_t *err, cudaStream_t st);
// One cache piece (reads r0 .. r0 + n_reads - 1, kc_off the piece's own); label, off and the ids are global.
void launch_kc_write(const uint64_t *kc_off, const uint64_t *kc_lo, const uint8_t *kc_hi, uint64_t r0, uint64_t n_reads,
                     int k, uint32_t lo, uint32_t hi, const uint32_t *label, const uint64_t *off, uint64_t *o_lo,
                     uint8_t *o_hi, uint32_t *o_id, cudaStream_t st);

// K2a: tuples per read in the bucket range [lo, hi).
void launch_enum_count(const uint8_t *fq, const ParsedReads &pr, int k, int min3, uint32_t lo, uint32_t hi,
                       uint32_t *cnt, uint32_t *err, cudaStream_t st);

// K2a for all scans at once (plain variant, at most 8 scans): cnt[s * stride + read] for the buckets
// [bounds[s], bounds[s+1]) (bounds: S + 1 device words).  Returns -1 (nothing launched) for other S.
int launch_enum_count_scans(const uint8_t *fq, const ParsedReads &pr, int k, const uint32_t *bounds, int S,
                            uint32_t *cnt, uint64_t stride, uint32_t *err, cudaStream_t st);

// K2b: tuples at off[read]: o_lo = kmer << 8 | adj, o_hi = kmer >> 56 (nullable when k <= 28),
// o_id = read id (scan 0, label == nullptr) or its component label.
void launch_enum_write(const uint8_t *fq, const ParsedReads &pr, int k, int min3, uint32_t lo, uint32_t hi,
                       const uint32_t *label, const uint64_t *off, uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id,
                       uint32_t *err, cudaStream_t st);

}  // namespace mp
