/* Shared helpers of the drop-in stage programs (genFastqIdx, genHistograms_metapart[min], metapart[min]). */
#ifndef MP_CLI_COMMON_H
#define MP_CLI_COMMON_H
#include <fcntl.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "metapart_gpu.h"

#define IDX_HDR 28u /* offset(8) offset2(8) readIdExtra(1) pad(3) readId(4) fileNo(4) */
#define UMAX32 4294967295ull

typedef struct {
    uint64_t offset, offset2;
    uint8_t extra;
    uint32_t read_id;
    int32_t file_no;
} idx_hdr;

static inline void cli_die(const char *prog, const char *what, int rc)
{
    fprintf(stderr, "%s: %s%s%s (code %d)\n", prog, what, rc ? ": " : "", rc ? mp_last_error() : "", rc);
    exit(1);
}

/* Read-only mapping of a whole file. */
static inline const char *map_file(const char *path, uint64_t *size)
{
    int fd = open(path, O_RDONLY);
    if (fd < 0) return NULL;
    struct stat st;
    if (fstat(fd, &st)) { close(fd); return NULL; }
    *size = (uint64_t)st.st_size;
    if (st.st_size == 0) { close(fd); return ""; }
    void *p = mmap(NULL, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
    close(fd);
    return p == MAP_FAILED ? NULL : (const char *)p;
}

static inline void hdr_put(unsigned char *r, const idx_hdr *h)
{
    memset(r, 0, IDX_HDR);
    memcpy(r + 0, &h->offset, 8);
    memcpy(r + 8, &h->offset2, 8);
    r[16] = h->extra;
    memcpy(r + 20, &h->read_id, 4);
    memcpy(r + 24, &h->file_no, 4);
}
static inline void hdr_get(const unsigned char *r, idx_hdr *h)
{
    memcpy(&h->offset, r + 0, 8);
    memcpy(&h->offset2, r + 8, 8);
    h->extra = r[16];
    memcpy(&h->read_id, r + 20, 4);
    memcpy(&h->file_no, r + 24, 4);
}

/* Headers of every record of an index file (.idx / .KmerIdx*); returns the record count or -1. */
static inline int read_index_headers(const char *path, idx_hdr **out)
{
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    fseek(f, 0, SEEK_END);
    long long sz = ftell(f);
    if (sz <= 0 || sz % MP_INDEX_RECORD_BYTES) { fclose(f); return -1; }
    int n = (int)(sz / MP_INDEX_RECORD_BYTES);
    *out = (idx_hdr *)calloc((size_t)n, sizeof(idx_hdr));
    unsigned char b[IDX_HDR];
    for (int i = 0; i < n; i++) {
        fseek(f, (long long)i * MP_INDEX_RECORD_BYTES, SEEK_SET);
        if (fread(b, 1, IDX_HDR, f) != IDX_HDR) { fclose(f); free(*out); return -1; }
        hdr_get(b, &(*out)[i]);
    }
    fclose(f);
    return n;
}

typedef struct {
    int nfiles;
    const char **data;
    uint64_t *size;
    uint64_t *base; /* byte offset of each file in the concatenation */
    uint64_t total;
} fastq_set;

static inline void load_fastq_set(const char *prog, int nfiles, char **names, fastq_set *fs)
{
    fs->nfiles = nfiles;
    fs->data = (const char **)calloc((size_t)nfiles, sizeof(char *));
    fs->size = (uint64_t *)calloc((size_t)nfiles, sizeof(uint64_t));
    fs->base = (uint64_t *)calloc((size_t)nfiles + 1, sizeof(uint64_t));
    fs->total = 0;
    for (int i = 0; i < nfiles; i++) {
        fs->data[i] = map_file(names[i], &fs->size[i]);
        if (!fs->data[i]) {
            fprintf(stderr, "%s: cannot open %s\n", prog, names[i]);
            exit(1);
        }
        fs->base[i] = fs->total;
        fs->total += fs->size[i];
    }
    fs->base[nfiles] = fs->total;
}

/* The files as one contiguous buffer (the mapping itself for a single file). */
static inline const char *fastq_concat(const fastq_set *fs, char **owned)
{
    *owned = NULL;
    if (fs->nfiles == 1) return fs->data[0];
    char *b = (char *)malloc(fs->total ? fs->total : 1);
    if (!b) return NULL;
    for (int i = 0; i < fs->nfiles; i++) memcpy(b + fs->base[i], fs->data[i], fs->size[i]);
    *owned = b;
    return b;
}

static inline int env_device(void)
{
    const char *d = getenv("MP_DEVICE");
    return d ? atoi(d) : 0;
}

#endif
