/*
 * genHistograms_metapart[min] kmerSize numPEFiles numSEFiles numInterleavedFiles file...
 *
 * Drop-in for the reference histogram stage (genHistograms.c:82-575) with the plain or
 * (built with -DMIN3) 3-minimizer count module.  Reads <file0>.idx, counts on the GPU
 * (mp_job_count) and writes <file0>.KmerIdx[_3min]<k> (the index records with read ids and
 * per-chunk bucket counts) and <file0>.kmerHist[_3min]<k> (1048577 exclusive prefix sums).
 */
#include "cli_common.h"

#ifdef MIN3
#define VARIANT "_3min"
#define IS_MIN3 1
#else
#define VARIANT ""
#define IS_MIN3 0
#endif

int main(int argc, char **argv)
{
    if (argc < 6) {
        printf("Usage: %s kmerSize numPEFiles numSEFiles numInterleavedFiles a.fastq ...\n", argv[0]);
        return 1;
    }
    const int k = atoi(argv[1]), npe = atoi(argv[2]), nse = atoi(argv[3]), nil = atoi(argv[4]);
    const int nfiles = argc - 5;
    if (npe) cli_die(argv[0], "two-file paired-end input is not supported", 0);
    if (nse + nil != nfiles || (nse && nil)) cli_die(argv[0], "file counts do not match the file list", 0);
    char path[4096];
    snprintf(path, sizeof path, "%s.idx", argv[5]);
    idx_hdr *h = NULL;
    const int nrec = read_index_headers(path, &h);
    if (nrec < 2) cli_die(argv[0], "cannot read the .idx file", 0);
    const int nchunks = nrec - 1;
    fastq_set fs;
    load_fastq_set(argv[0], nfiles, &argv[5], &fs);
    uint64_t *starts = (uint64_t *)calloc((size_t)nrec, sizeof(uint64_t));
    for (int i = 0; i < nrec; i++) {
        if (h[i].file_no < 0 || h[i].file_no >= nfiles) cli_die(argv[0], "index record names a missing file", 0);
        starts[i] = fs.base[h[i].file_no] + h[i].offset;
    }
    char *owned = NULL;
    const char *buf = fastq_concat(&fs, &owned);
    mp_ctx *ctx = NULL;
    mp_job *job = NULL;
    int rc = mp_ctx_create(env_device(), 0, &ctx);
    if (rc) cli_die(argv[0], "no GPU context", rc);
    if ((rc = mp_job_create(ctx, &job))) cli_die(argv[0], "job", rc);
    mp_job_set_kmer_cache(job, 0); /* this process only counts */
    if ((rc = mp_job_load_fastq(job, buf, fs.total, fs.size, nfiles, nil > 0))) cli_die(argv[0], "loading reads", rc);
    uint64_t *hist = (uint64_t *)calloc(MP_NUM_BUCKETS + 1, sizeof(uint64_t));
    uint32_t *counts = (uint32_t *)calloc((size_t)nchunks * MP_NUM_BUCKETS, sizeof(uint32_t));
    uint64_t *reads = (uint64_t *)calloc((size_t)nchunks, sizeof(uint64_t));
    if (!hist || !counts || !reads) cli_die(argv[0], "out of host memory", 0);
    if ((rc = mp_job_count(job, k, IS_MIN3, starts, nchunks, hist, counts, reads))) cli_die(argv[0], "counting", rc);
    /* .KmerIdx: index headers with cumulative read ids (genHistograms.c:280-291) and bucket counts */
    snprintf(path, sizeof path, "%s.KmerIdx%s%d", argv[5], VARIANT, k);
    FILE *out = fopen(path, "wb");
    if (!out) cli_die(argv[0], "cannot write the .KmerIdx file", 0);
    unsigned char *rec = (unsigned char *)calloc(1, MP_INDEX_RECORD_BYTES);
    uint64_t acc = 0;
    for (int i = 0; i < nrec; i++) {
        idx_hdr x = h[i];
        if (i > 0) {
            acc += reads[i - 1];
            if (acc / UMAX32 >= 256) cli_die(argv[0], "too many reads", 0);
            x.read_id = (uint32_t)(acc % UMAX32);
            x.extra = (uint8_t)(acc / UMAX32);
        }
        memset(rec, 0, MP_INDEX_RECORD_BYTES);
        hdr_put(rec, &x);
        if (i < nchunks) memcpy(rec + IDX_HDR, counts + (size_t)i * MP_NUM_BUCKETS, MP_NUM_BUCKETS * sizeof(uint32_t));
        if (fwrite(rec, 1, MP_INDEX_RECORD_BYTES, out) != MP_INDEX_RECORD_BYTES) cli_die(argv[0], "short write", 0);
    }
    fclose(out);
    snprintf(path, sizeof path, "%s.kmerHist%s%d", argv[5], VARIANT, k);
    out = fopen(path, "wb");
    if (!out || fwrite(hist, sizeof(uint64_t), MP_NUM_BUCKETS + 1, out) != MP_NUM_BUCKETS + 1)
        cli_die(argv[0], "cannot write the .kmerHist file", 0);
    fclose(out);
    double ms[8];
    mp_job_stage_ms(job, ms, 8);
    printf("[0]TOTALKMERS %llu, TOTALREADS %llu (GPU parse %.3f ms, count %.3f ms)\n", (unsigned long long)hist[MP_NUM_BUCKETS],
           (unsigned long long)mp_job_num_reads(job), ms[0], ms[1]);
    mp_job_destroy(job);
    mp_ctx_destroy(ctx);
    free(owned);
    return 0;
}
