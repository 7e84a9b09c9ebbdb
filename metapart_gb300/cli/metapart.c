/*
 * metapart[min] -o outPrefix fastqBufferSize kmerSize numScans numThreads numPEFiles numSEFiles
 *               numInterleavedFiles file...
 *
 * Drop-in for the reference partitioner (metapart.c:3544-4150): reads <file0>.KmerIdx[_3min]<k>
 * and <file0>.kmerHist[_3min]<k>, partitions the reads on the GPU (mp_job_partition) and writes
 * <outPrefix>/Rank0/FromTid<t>_ToRank<p>.paired.fastq for t < numThreads, p < 16.
 * MP_DUMP_DIR=<dir> writes the reference-format stage dumps used by the parity tests.
 */
#include <getopt.h>

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
    static struct option longopts[] = {{"out-prefix", required_argument, 0, 'o'}, {0, 0, 0, 0}};
    const char *oprefix = ".";
    int c;
    while ((c = getopt_long(argc, argv, "o:", longopts, NULL)) != -1)
        if (c == 'o') oprefix = optarg;
    char **a = &argv[optind - 1];
    const int na = argc - (optind - 1);
    if (na < 9) {
        printf("Usage: %s -o <output-prefix> fastqBufferSize kmerSize numScans numThreads numPEFiles numSEFiles "
               "numInterleavedFiles a.fastq ...\n", argv[0]);
        return 1;
    }
    const uint64_t bufsize = strtoull(a[1], NULL, 10);
    mp_part_params p;
    p.k = atoi(a[2]);
    p.num_scans = atoi(a[3]);
    p.num_threads = atoi(a[4]);
    p.min3 = IS_MIN3;
    const int npe = atoi(a[5]), nse = atoi(a[6]), nil = atoi(a[7]);
    const int nfiles = na - 8;
    char **files = &a[8];
    if (npe) cli_die(argv[0], "two-file paired-end input is not supported", 0);
    if (nse + nil != nfiles || (nse && nil)) cli_die(argv[0], "file counts do not match the file list", 0);
    char path[4096];
    snprintf(path, sizeof path, "%s.KmerIdx%s%d", files[0], VARIANT, p.k);
    idx_hdr *h = NULL;
    const int nrec = read_index_headers(path, &h);
    if (nrec < 2) cli_die(argv[0], "cannot read the .KmerIdx file", 0);
    const int nchunks = nrec - 1;
    uint64_t *hist = (uint64_t *)calloc(MP_NUM_BUCKETS + 1, sizeof(uint64_t));
    snprintf(path, sizeof path, "%s.kmerHist%s%d", files[0], VARIANT, p.k);
    FILE *fh = fopen(path, "rb");
    if (!fh || fread(hist, sizeof(uint64_t), MP_NUM_BUCKETS + 1, fh) != MP_NUM_BUCKETS + 1)
        cli_die(argv[0], "cannot read the .kmerHist file", 0);
    fclose(fh);
    fastq_set fs;
    load_fastq_set(argv[0], nfiles, files, &fs);
    uint64_t *starts = (uint64_t *)calloc((size_t)nrec, sizeof(uint64_t));
    uint64_t *first = (uint64_t *)calloc((size_t)nrec, sizeof(uint64_t));
    for (int i = 0; i < nrec; i++) {
        if (h[i].file_no < 0 || h[i].file_no >= nfiles) cli_die(argv[0], "index record names a missing file", 0);
        starts[i] = fs.base[h[i].file_no] + h[i].offset;
        first[i] = (uint64_t)h[i].extra * UMAX32 + h[i].read_id;
        /* loadChunk asserts that a chunk fits the FASTQ buffer (metapart.c:471) */
        if (i > 0 && starts[i] - starts[i - 1] >= bufsize) cli_die(argv[0], "fastqBufferSize is smaller than a chunk", 0);
    }
    char *owned = NULL;
    const char *buf = fastq_concat(&fs, &owned);
    mp_ctx *ctx = NULL;
    mp_job *job = NULL;
    int rc = mp_ctx_create(env_device(), 0, &ctx);
    if (rc) cli_die(argv[0], "no GPU context", rc);
    if ((rc = mp_job_create(ctx, &job))) cli_die(argv[0], "job", rc);
    if (getenv("MP_DUMP_DIR")) mp_job_set_dump_dir(job, getenv("MP_DUMP_DIR"));
    if ((rc = mp_job_load_fastq(job, buf, fs.total, fs.size, nfiles, nil > 0))) cli_die(argv[0], "loading reads", rc);
    uint64_t bounds[17];
    if ((rc = mp_job_partition(job, &p, starts, first, nchunks, hist, bounds))) cli_die(argv[0], "partitioning", rc);
    const int nout = 16 * p.num_threads;
    uint64_t *sizes = (uint64_t *)calloc((size_t)nout, sizeof(uint64_t));
    uint64_t total = 0;
    if ((rc = mp_job_output(job, NULL, 0, sizes, &total))) cli_die(argv[0], "output", rc);
    char *out = (char *)malloc(total ? total : 1);
    if (!out) cli_die(argv[0], "out of host memory", 0);
    if ((rc = mp_job_output(job, out, total, sizes, &total))) cli_die(argv[0], "output", rc);
    uint64_t pos = 0;
    for (int j = 0; j < nout; j++) {
        const int pid = j / p.num_threads, tid = j % p.num_threads;
        snprintf(path, sizeof path, "%s/Rank0/FromTid%d_ToRank%d.paired.fastq", oprefix, tid, pid);
        FILE *fo = fopen(path, "wb");
        if (!fo) cli_die(argv[0], "cannot write an output file (does <out>/Rank0 exist?)", 0);
        if (sizes[j] && fwrite(out + pos, 1, sizes[j], fo) != sizes[j]) cli_die(argv[0], "short write", 0);
        fclose(fo);
        pos += sizes[j];
    }
    double ms[8];
    mp_job_stage_ms(job, ms, 8);
    printf("[0] GPU ms: parse %.3f, enumerate %.3f, sort %.3f, filter %.3f, unionFind %.3f, mate union+plan %.3f, output %.3f\n",
           ms[0], ms[2], ms[3], ms[4], ms[5], ms[6], ms[7]);
    printf("[0] partitions:");
    for (int i = 0; i <= 16; i++) printf(" %llu", (unsigned long long)bounds[i]);
    printf("\n");
    mp_job_destroy(job);
    mp_ctx_destroy(ctx);
    free(out);
    free(owned);
    return 0;
}
