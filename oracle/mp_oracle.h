/*
 * CPU restatement of the MetaPart read-partitioning path (test infrastructure:
 * the checker for the GPU implementation and the timed CPU baseline; never part
 * of the product).  Three entry points mirror the reference stage programs and
 * read/write the same files:
 *
 *   mpo_fastq_index     <-> genFastqIdx main        (genFastqIdx.c:142-376)
 *   mpo_gen_histograms  <-> genHistograms main      (genHistograms.c:82-575)
 *   mpo_metapart        <-> metapart main           (metapart.c:3544-4150)
 *
 * With MP_DUMP_DIR set, mpo_metapart writes the same stage dumps as the
 * reference built through oracle/ref_hooks.c (scan<s>_enum.bin, ... ).
 * All return 0 on success and a negative MPO_E* code otherwise.
 */
#ifndef MP_ORACLE_H
#define MP_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum {
    MPO_OK = 0,
    MPO_EARG = -1,   /* invalid argument (k, thread count, file kinds, ...) */
    MPO_EIO = -2,    /* file could not be read or written */
    MPO_EFMT = -3,   /* malformed FASTQ or index file */
    MPO_ENOMEM = -4,
    MPO_EUNSUP = -5  /* configuration the reference itself mishandles */
};

int mpo_fastq_index(int num_chunks, int n_pe, int n_se, int n_il, int nfiles, const char *const *files);
int mpo_gen_histograms(int k, int min3, int n_pe, int n_se, int n_il, int nfiles, const char *const *files);
int mpo_metapart(const char *out_prefix, uint64_t fastq_buffer_size, int k, int num_scans, int num_threads,
                 int min3, int n_pe, int n_se, int n_il, int nfiles, const char *const *files);
const char *mpo_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
