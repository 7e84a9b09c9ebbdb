/*
 * metapart_gpu.h -- C ABI of the GB300 read-partitioning path (libmetapart_gpu.so).
 *
 * The reference (MetaPart) exposes this path as three stage programs that talk
 * through files, plus a link-time k-mer module.  Each entry point below names
 * the reference interface it replaces.  Plain pointers and sizes only; host
 * buffers are caller-owned, device memory is owned by the job.  Every call
 * returns 0 or a negative MP_E* code (never aborts); mp_last_error() gives the
 * message of the calling thread's last failure.
 *
 * Limits (the reference's own, made explicit): k in [11, 31]; m is 10
 * (4^10 buckets); read ids below 2^32 - 1; an even read count for the mate
 * union; metapart reads shorter than 300 + k; the 3-minimizer variant with
 * numScans == 1; single-end or interleaved input (no two-file paired end).
 */
#ifndef METAPART_GPU_H
#define METAPART_GPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define MP_OK 0
#define MP_EARG (-1)      /* invalid argument */
#define MP_EIO (-2)       /* file read/write failed */
#define MP_EFMT (-3)      /* malformed FASTQ / index / histogram */
#define MP_ENOMEM (-4)    /* host or device allocation failed, or HBM budget exceeded */
#define MP_EUNSUP (-5)    /* configuration outside the supported limits */
#define MP_ECUDA (-6)     /* CUDA runtime error */
#define MP_EDEVICE (-7)   /* a kernel's bounded wait or capacity check failed */

#define MP_NUM_BUCKETS 1048576u   /* 4^10 */
#define MP_INDEX_RECORD_BYTES 4194344u
#define MP_NUM_OUT_PARTITIONS 16

typedef struct mp_ctx mp_ctx;
typedef struct mp_job mp_job;

/* Thread-local message of the last failed call. */
const char *mp_last_error(void);

/* One context per device: stream pool, HBM budget accounting.  Jobs, batches and servers keep a pointer
 * to their context: destroy it only after all of them are destroyed. */
int mp_ctx_create(int device, uint64_t hbm_budget_bytes, mp_ctx **out);
void mp_ctx_destroy(mp_ctx *ctx);
uint64_t mp_ctx_hbm_in_use(const mp_ctx *ctx);

/* Chunk index of FASTQ files in memory.
 * Replaces genFastqIdx main (genFastqIdx.c:142-376) and getFileIndex (:28-53).
 * files[i]/sizes[i]: file contents; out_offsets receives (fileNo, offset) pairs of
 * up to num_chunks+1 index records (last = end sentinel); *out_count their number. */
int mp_fastq_index(int num_chunks, int n_pe, int n_se, int n_il, int nfiles, const char *const *files,
                   const uint64_t *sizes, int32_t *out_file_no, uint64_t *out_offsets, int *out_count);

/* A partition job: reads resident in HBM plus all stage state, on its own stream. */
int mp_job_create(mp_ctx *ctx, mp_job **out);
void mp_job_destroy(mp_job *job);

/* Upload and parse FASTQ on the GPU (records of header, sequence, '+', quality).
 * Replaces the per-chunk FASTQ walks getNextRead (genHistograms.c:60-80, metapart.c:296-369),
 * loadChunk (metapart.c:371-500) and getNextFullRead (metapart.c:211-294).
 * bytes: the files concatenated; file_sizes: each file's length (each ends on a record end). */
int mp_job_load_fastq(mp_job *job, const char *bytes, uint64_t nbytes, const uint64_t *file_sizes, int nfiles,
                      int interleaved);
/* Same, for bytes already in device memory (copied into the job). */
int mp_job_load_fastq_device(mp_job *job, const void *dev_bytes, uint64_t nbytes, const uint64_t *file_sizes,
                             int nfiles, int interleaved);
/* Same, using bytes already in device memory in place (no copy): they must start on a 16-byte boundary,
 * be followed by 64 readable bytes, and stay unchanged until the job is reset or destroyed.  For a caller
 * whose reads are already in HBM; no counterpart in the reference. */
int mp_job_load_fastq_device_inplace(mp_job *job, const void *dev_bytes, uint64_t nbytes, const uint64_t *file_sizes,
                                     int nfiles, int interleaved);
uint64_t mp_job_num_reads(const mp_job *job);

/* Releases the job's reads and stage state (device memory) and keeps its stream, so one job can
 * run many inputs back to back.  No reference counterpart (the reference runs one input per process). */
int mp_job_reset(mp_job *job);

/* The job's CUDA stream (cudaStream_t), for callers that order their own work or events around it. */
void *mp_job_stream(mp_job *job);

/* Number of kernels this library has launched in the process (instrumentation). */
uint64_t mp_launch_count(void);

/* m-mer histogram and per-chunk bucket counts of the loaded reads.
 * Replaces genHistograms main (genHistograms.c:82-575) with the count module
 * getCanonKmers/getMmerPrefix (countMmers.c:60-217; countMmers_3minimizers.c:83-271).
 * chunk_starts: nchunks+1 absolute byte offsets (record starts; last = end of input).
 * hist_out: 1048577 exclusive prefix sums (the .kmerHist layout, genHistograms.c:325-342);
 * chunk_counts_out (nullable): nchunks x 1048576 bucket counts (fileIndex.kmerFreqCount);
 * chunk_reads_out (nullable): reads per chunk. */
int mp_job_count(mp_job *job, int k, int min3, const uint64_t *chunk_starts, int nchunks, uint64_t *hist_out,
                 uint32_t *chunk_counts_out, uint64_t *chunk_reads_out);

/* mp_job_load_fastq followed by mp_job_count (without per-chunk bucket counts), with the upload
 * overlapped: for pinned host bytes and the plain variant, the input goes up in segments of whole
 * chunks on a second stream while the job's stream parses and counts the segments already in HBM.
 * Results, errors and the job state afterwards are those of the two calls made one after the other
 * (which is also what runs for pageable bytes, the 3-minimizer variant, or when a segment fails).
 * The reference reads each chunk from disk inside genHistograms' count loop (genHistograms.c:82-575);
 * this has no further counterpart there. */
int mp_job_load_count(mp_job *job, const char *bytes, uint64_t nbytes, const uint64_t *file_sizes, int nfiles,
                      int interleaved, int k, int min3, const uint64_t *chunk_starts, int nchunks, uint64_t *hist_out,
                      uint64_t *chunk_reads_out);
/* Pieces the job's k-mer cache is held in: 0 (no cache), 1 (mp_job_count), or one per upload segment
 * of mp_job_load_count.  Tracing only; no counterpart in the reference. */
int mp_job_kmer_cache_pieces(const mp_job *job);

typedef struct {
    int k;            /* kmerSize */
    int min3;         /* 1: 3-minimizer variant (enumerateKmers_3minimizers.c) */
    int num_scans;    /* numScans: semantic passes over the m-mer space */
    int num_threads;  /* numThreads: chunk-to-thread map, k-mer thread ranges, output file split */
} mp_part_params;

/* Read partitioning: enumerate -> stable sort -> mischief filter -> union-find per scan,
 * then mate union and the 16 work partitions.
 * Replaces metapart main (metapart.c:3544-4100): generateKmersInScan (:1192), sortKmerList (:1852),
 * markMischiefKmers (:2270), unionFindPar2 (:2520), unionFind (:2736), printStats (:3227),
 * unionFindPeReads (:2801), the work-partition planner (:4016-4053), and the enum module
 * getCanonKmers (enumerateKmers.c:127; enumerateKmers_3minimizers.c:129).
 * chunk_first_read: nchunks+1 read ids (fileIndex readId/readIdExtra; last = read count).
 * hist: the 1048577-entry .kmerHist of the same k and variant.  bounds_out: 17 read-id bounds. */
int mp_job_partition(mp_job *job, const mp_part_params *p, const uint64_t *chunk_starts,
                     const uint64_t *chunk_first_read, int nchunks, const uint64_t *hist, uint64_t *bounds_out);

/* Final component label (root read id) of every read after mp_job_partition (the reference's
 * compressed parent array, metapart.c:4026-4030).  out: mp_job_num_reads() entries. */
int mp_job_labels(mp_job *job, uint32_t *out);

/* Partition FASTQ output, grouped by file j = partition * num_threads + tid in the order of the
 * reference's FromTid<tid>_ToRank<partition>.paired.fastq files.
 * Replaces writeOutput3 (metapart.c:956-1066).  With out == NULL only file_sizes/total are filled (the
 * files' layout is planned, no bytes move).  With out, the files are built in HBM in batches, each
 * batch copied down while the next is built. */
int mp_job_output(mp_job *job, char *out, uint64_t capacity, uint64_t *file_sizes, uint64_t *total);

/* The same files built in HBM (kept by the job until it is reset or partitions again): *d_out their
 * device address.  For a caller that consumes them on the GPU; no counterpart in the reference. */
int mp_job_output_device(mp_job *job, const void **d_out, uint64_t *file_sizes, uint64_t *total);

/* Stable sort of k-mer tuples by (k-mer, adjacency byte) on the device (onesweep LSD radix sort).
 * Replaces radixPass and the range-partition + 9-pass driver of sortKmerList (metapart.c:1494-1598,
 * 1852-2200).  All pointers are device pointers: lo = kmer << 8 | adj, hi = kmer >> 56 (both NULL when
 * 2k + 8 <= 64), id = read id.  Ties keep input order.  Scratch comes from the context's stream-ordered
 * pool; the call returns after the sort completed on `stream` (a cudaStream_t, NULL = legacy stream). */
int mp_sort_tuples(mp_ctx *ctx, const uint64_t *lo_in, const uint8_t *hi_in, const uint32_t *id_in, uint64_t *lo_out,
                   uint8_t *hi_out, uint32_t *id_out, uint64_t n, void *stream);

/* Allocation-free variant of mp_sort_tuples, for callers that cannot allocate device memory while
 * they run: a host that gives this library only buffers from its own device allocator, or a loop that
 * must not call cudaMalloc/cudaFree (they can synchronize the whole device) between its steps.  Same
 * arguments and results as mp_sort_tuples, without a context; it returns after the sort completed on
 * `stream`.  Each output array may be its own input array (sorted in place); an output that overlaps any
 * other input, or its own input only in part, returns MP_EARG.  It allocates nothing: its scratch is one
 * fixed device array inside the library (about 14 MB on every GPU that loads the library, held until the
 * process exits), so n is limited to 1,048,576 tuples -- a larger n returns MP_EARG before any GPU work.
 * The first call on a device looks up that array's device address (cudaGetSymbolAddress); make that
 * first call before any stream capture.  Every call uses the same array: calls that overlap on the GPU
 * (other streams, other host threads) race on it and corrupt each other.  This entry point has no
 * counterpart in the reference. */
int mp_sort_tuples_noalloc(const uint64_t *lo_in, const uint8_t *hi_in, const uint32_t *id_in, uint64_t *lo_out,
                           uint8_t *hi_out, uint32_t *id_out, uint64_t n, void *stream);

/* ---- Batches: many independent samples partitioned together.
 * The reference partitions one input per process launch (metapart.c:3544-4150); this has no counterpart
 * there.  Every sample gets exactly what mp_job_partition + mp_job_output give it alone with numScans = 1
 * and the plain variant: the same 16 bounds, component labels and partition files.  The samples share
 * the stages -- one upload of their bytes one after another, per-sample m-mer histograms and scan plans
 * computed on the device, one enumeration, one sort of every sample's tuples (the sample is the most
 * significant part of the key), one filter and union sweep over every sample's thread ranges, one mate
 * union, one output gather -- in groups of samples sized to the context's HBM budget. */
typedef struct mp_batch mp_batch;

typedef struct {
    int k;            /* kmerSize of every sample */
    int interleaved;  /* 1: every sample is interleaved pairs, 0: every sample is single end */
} mp_batch_params;

typedef struct {
    const char *fastq;     /* one FASTQ file (pinned host memory lets its upload overlap other work) */
    uint64_t nbytes;
    int num_chunks;        /* genFastqIdx chunks */
    int num_threads;       /* numThreads: a divisor of the chunk count, at most 256 */
    char *out;             /* nullable: the partition files, grouped as mp_job_output */
    uint64_t out_cap;
    uint64_t *file_sizes;  /* nullable: 16 x num_threads file sizes */
    uint32_t *labels;      /* nullable: the component label of every read (the sample's own ids) */
    uint64_t labels_cap;
} mp_batch_sample;

typedef struct {
    int status;            /* 0 or a negative MP_E* code */
    char error[256];
    uint64_t n_reads;
    uint64_t out_total;    /* partition FASTQ bytes */
    uint64_t bounds[17];   /* the 16 work partitions' read-id bounds */
} mp_batch_result;

int mp_batch_create(mp_ctx *ctx, mp_batch **out);
void mp_batch_destroy(mp_batch *b);
/* Partitions every sample; returns the first failure (its message names the sample), results[] per sample. */
int mp_batch_run(mp_batch *b, const mp_batch_params *p, int nsamples, const mp_batch_sample *samples,
                 mp_batch_result *results);
/* Device ms of the last run per stage, summed over its groups (the order of mp_job_stage_ms). */
int mp_batch_stage_ms(const mp_batch *b, double *ms, int n);
/* Groups the last run went in. */
int mp_batch_groups(const mp_batch *b);
/* The batch's bounded device waits, as mp_job_set_wait_limits. */
int mp_batch_set_wait_limits(mp_batch *b, uint32_t lookback_spins, uint32_t union_retries, uint32_t mate_rounds);
/* The last run's bucket-digit sort passes: tuples, passes, device ms and algorithmic bytes. */
int mp_batch_sort_stats(const mp_batch *b, uint64_t *tuples, int *passes, double *pass_ms, uint64_t *bytes);

/* ---- Request loop: continuous admission of partition jobs on one context.
 * The reference runs one input per MPI launch; this loop has no counterpart there.  Worker threads
 * each own one job (one CUDA stream); a request is admitted in arrival order when a worker is free
 * and its estimated HBM footprint fits in what the server budget has left, so the stages of
 * different jobs overlap on the GPU.  A job that runs out of device memory beside others is run
 * again alone.  Each admitted request runs the whole chain: chunk index (genFastqIdx), upload,
 * m-mer histogram (genHistograms), partition (metapart) and the partition FASTQ download. */
typedef struct mp_server mp_server;

typedef struct {
    int k, min3, num_scans, num_threads;  /* as mp_part_params */
    int num_chunks;                       /* genFastqIdx chunks; a multiple of num_threads */
    int interleaved;                      /* 1: interleaved pairs, 0: single end */
    int read_store;                       /* MP_STORE_*: what the request's count pass keeps for its partition
                                             (MP_STORE_PACKED admits the most requests at once: 0.375 bytes per
                                             base against the k-mer cache's 9 per position) */
} mp_request_params;

typedef struct {
    int status;            /* 0 or a negative MP_E* code */
    char error[256];       /* message when status != 0 */
    uint64_t n_reads;
    uint64_t out_total;    /* partition FASTQ bytes written to the request's out buffer */
    uint64_t bounds[17];   /* the 16 work partitions' read-id bounds */
    uint64_t footprint;    /* HBM bytes reserved at admission */
    double t_submit_ms, t_admit_ms, t_done_ms;  /* since the server was created */
    double device_ms;      /* sum of the job's stage times on the GPU */
} mp_result;

typedef struct {
    uint64_t queued, admitted, completed, reserved, peak_reserved, budget;
    int running, peak_running;
} mp_server_stats_t;

/* Estimated device bytes of one request (FASTQ, read table, forest, the largest scan's tuple
 * buffers, output, the store of the reads its count pass keeps), from the request size and its first
 * records. */
uint64_t mp_request_footprint(const char *fastq, uint64_t nbytes, const mp_request_params *p);

/* slots: worker threads (jobs in flight at most); hbm_budget: bytes the admitted footprints may add
 * up to (0 = unlimited; the context's own budget still bounds the real allocations). */
int mp_server_create(mp_ctx *ctx, int slots, uint64_t hbm_budget, mp_server **out);

/* Queues one request.  fastq (one single-end or interleaved FASTQ) and the output buffers stay
 * owned by the caller and must stay valid until the request is done; out receives the partition
 * files grouped as in mp_job_output, file_sizes (nullable) 16 x num_threads sizes, labels (nullable,
 * labels_cap entries) the component label of every read. */
int mp_server_submit(mp_server *s, const char *fastq, uint64_t nbytes, const mp_request_params *p, char *out,
                     uint64_t out_cap, uint64_t *file_sizes, uint32_t *labels, uint64_t labels_cap, uint64_t *ticket);

/* 1 and *res when the request is done (its result is then released), 0 while it is pending; with
 * wait != 0 blocks until done.  MP_EARG for a ticket never issued or whose result was released already
 * (also to a second thread waiting on the same ticket when the first takes the result). */
int mp_server_poll(mp_server *s, uint64_t ticket, int wait, mp_result *res);
int mp_server_stats(mp_server *s, mp_server_stats_t *st);

/* Runs the queued requests to completion, then stops the workers. */
void mp_server_destroy(mp_server *s);

/* k-mer cache (default on): mp_job_count of the plain variant keeps every read position's canonical
 * k-mer and adjacency byte (9 bytes per position) in the job, and the next mp_job_partition with the
 * same k filters it per scan instead of recomputing k-mers from the reads; the partition releases it.
 * Skipped without error when device memory or the budget does not allow it.  Turn it off for a
 * count-only job (the drop-in genHistograms).  No counterpart in the reference, whose stages are
 * separate processes. */
int mp_job_set_kmer_cache(mp_job *job, int enable);

/* What the count pass of the plain variant keeps of the reads for the next mp_job_partition of the same k
 * (mp_job_count, mp_job_load_count):
 *   MP_STORE_KMER_CACHE (default): every position's canonical k-mer and adjacency byte, 9 bytes per
 *     position (21.6 GB for 20M reads of 150 bp); the partition's enumeration only filters it;
 *   MP_STORE_PACKED: the reads 2 bits per base with an N mask, 0.375 bytes per base (1.1 GB for the same
 *     reads); the enumeration recomputes the k-mers from them, so it takes longer;
 *   MP_STORE_FASTQ: nothing; the enumeration recomputes the k-mers from the FASTQ bytes.
 * An input with any sequence byte other than A, C, G, T, N keeps no packed copy (the FASTQ path runs); a
 * store that does not fit the budget or the device is skipped.  mp_job_set_kmer_cache(job, 1 / 0) is
 * MP_STORE_KMER_CACHE / MP_STORE_FASTQ.  mp_job_read_store tells which store the job holds now.  No
 * counterpart in the reference, whose stages are separate processes that re-read the FASTQ files. */
#define MP_STORE_FASTQ 0
#define MP_STORE_KMER_CACHE 1
#define MP_STORE_PACKED 2
int mp_job_set_read_store(mp_job *job, int store);
int mp_job_read_store(const mp_job *job);

/* Most tuples one scan of mp_job_partition holds in HBM at once (0, the default: what the context's
 * budget, or the device, has left at about 32 bytes per tuple; the environment variable
 * MP_SCAN_PIECE_TUPLES overrides both).  A scan of the plain variant with more tuples runs in pieces of
 * consecutive m-mer buckets, swept twice (sort and mischief filter of every piece, then sort and union of
 * every piece), with the same results as the whole scan at once.  The reference has no counterpart: its
 * scans are what bounds its memory (numScans, metapart.c:3720-3791), and a different numScans changes
 * the partitions; pieces inside a scan do not. */
int mp_job_set_scan_piece_tuples(mp_job *job, uint64_t max_tuples);
/* Iteration limits of the job's bounded device waits (0 keeps the default): the sort's decoupled
 * look-back polls of one predecessor's status word (default 2^22), the union-find's hook retries of one
 * union (2^20), and the mate union's rounds (4,000,000).  A wait that runs out makes the call return
 * MP_EDEVICE with a message naming it; the job's results are then undefined, the context stays usable
 * and a reset job runs normally.  The reference's own loops are unbounded (its edge replay,
 * metapart.c:2736-2800); these limits have no counterpart there. */
int mp_job_set_wait_limits(mp_job *job, uint32_t lookback_spins, uint32_t union_retries, uint32_t mate_rounds);

/* Self-checks of the job's intermediate results (off by default; the environment variable MP_CHECK=1
 * turns them on for every job): after every scan's sort (or every piece's), that no adjacent tuple pair is
 * out of (k-mer, adjacency) order; after the mate union, that every read's parent is a root or BAD.  A
 * failed check makes mp_job_partition return MP_EDEVICE naming it.  The reference checks neither. */
int mp_job_set_checks(mp_job *job, int on);

/* Adjacent pairs out of (k-mer, adjacency) order in a device tuple array (lo and hi as mp_sort_tuples;
 * hi NULL when 2k + 8 <= 64) into *out: 0 for a sorted array.  Returns after the count on `stream`. */
int mp_count_unsorted(mp_ctx *ctx, const uint64_t *lo, const uint8_t *hi, uint64_t n, void *stream, uint64_t *out);

/* Bucket-range pieces the last mp_job_partition ran its scans in, summed over the scans (numScans when
 * no scan was split).  Tracing only. */
int mp_job_scan_pieces(const mp_job *job);

/* Optional stage dumps in the reference's formats (the files oracle/ref_hooks.c writes),
 * for parity testing.  NULL disables; with the environment variable MP_DUMP_TUPLES=0 only the
 * per-read dumps (BAD flags, parents, sizes) are written, not the tuple streams. */
int mp_job_set_dump_dir(mp_job *job, const char *dir);

/* Device time of the last count/partition/output calls per stage, in ms:
 * [0] parse [1] count [2] enumerate [3] sort [4] filter [5] union-find [6] mate union+partition [7] output. */
int mp_job_stage_ms(const mp_job *job, double *ms, int n);

/* Algorithmic bytes and device time of the last sort's digit passes (roofline reporting). */
int mp_job_sort_stats(const mp_job *job, uint64_t *tuples, int *passes, double *pass_ms, uint64_t *bytes);

/* Where the last partition's sort time went, summed over its scans: the m-mer bucket digit passes, the
 * shared-memory sort of bucket units, and the buckets too large for a unit (ms, and their counts);
 * unit_counters (nullable, 11 entries): [0] the unit sort's digit passes, [1..3] its SM cycles in the load,
 * digit-pass and store phases, each summed over units; [4..8] the bucket digit passes' SM cycles in the
 * tile-id fetch, loads and ranks, digit scan, tile order and look-back, and stores, each summed over
 * tiles; [9] [10] the status words digit 0's look-back read and its polls of words not yet posted.
 * Tracing only; no counterpart in the reference. */
int mp_job_sort_split(const mp_job *job, double *pass_ms, double *unit_ms, double *big_ms, uint64_t *units,
                      uint64_t *big_buckets, uint64_t *big_tuples, uint64_t *unit_counters);

#ifdef __cplusplus
}
#endif
#endif
