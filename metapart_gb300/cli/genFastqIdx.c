/*
 * genFastqIdx numPartitions numPEFiles numSEFiles numInterleavedFiles file...
 *
 * Drop-in for the reference chunk indexer (genFastqIdx.c:142-376): writes
 * <file0>.idx with numPartitions (+1 sentinel) index records of 4,194,344 bytes.
 * Host-only: a few 3 KB boundary searches, no GPU work.
 */
#include "cli_common.h"

int main(int argc, char **argv)
{
    if (argc < 6) {
        printf("Usage: %s numPartitions numPEFiles numSEFiles numInterleavedFiles a.fastq ...\n", argv[0]);
        return 1;
    }
    const int chunks = atoi(argv[1]), npe = atoi(argv[2]), nse = atoi(argv[3]), nil = atoi(argv[4]);
    const int nfiles = argc - 5;
    fastq_set fs;
    load_fastq_set(argv[0], nfiles, &argv[5], &fs);
    int32_t *fno = (int32_t *)calloc((size_t)chunks + 1, sizeof(int32_t));
    uint64_t *ofs = (uint64_t *)calloc((size_t)chunks + 1, sizeof(uint64_t));
    int n = 0;
    int rc = mp_fastq_index(chunks, npe, nse, nil, nfiles, fs.data, fs.size, fno, ofs, &n);
    if (rc) cli_die(argv[0], "indexing failed", rc);
    char path[4096];
    snprintf(path, sizeof path, "%s.idx", argv[5]);
    FILE *out = fopen(path, "wb");
    if (!out) cli_die(argv[0], "cannot write the index file", 0);
    unsigned char *rec = (unsigned char *)calloc(1, MP_INDEX_RECORD_BYTES);
    for (int i = 0; i < n; i++) {
        idx_hdr h = {ofs[i], 0, 0, 0, fno[i]};
        hdr_put(rec, &h);
        if (fwrite(rec, 1, MP_INDEX_RECORD_BYTES, out) != MP_INDEX_RECORD_BYTES) cli_die(argv[0], "short write", 0);
    }
    fclose(out);
    printf("%s: %d index records written to %s\n", argv[0], n, path);
    return 0;
}
