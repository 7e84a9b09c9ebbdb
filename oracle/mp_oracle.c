/*
 * CPU restatement of the MetaPart read-partitioning path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker the GPU implementation is compared
 * against, and the CPU baseline the benchmark times.  Nothing in the product
 * links or calls this file.  Each function cites the reference lines it
 * restates; the restatement is pinned against the reference binaries built by
 * oracle/build_ref.sh (tests/test_oracle_vs_reference.py) and against the
 * committed golden digests (tests/golden/).
 *
 * Semantics notes (all follow the reference at one MPI rank):
 *  - m is 10: 4^10 buckets, index records of 4,194,344 bytes.
 *  - k in [11, 31]; the tuple keeps the low 64 bits of the k-mer code.
 *  - read ids are below 2^32 - 1, so the 5-byte parent encoding has quotient 0
 *    except for the BAD marker 0xBADBADBAD (quotient 11, rem 0xADBADBB8).
 *  - union-find runs the reference's per-thread edge sweeps one thread range
 *    after another, which is one of the interleavings the reference's racy
 *    parallel hooking converges to (its edge replay, metapart.c:2736-2800,
 *    repairs lost hooks); the resulting partition is the connected components
 *    of the run edges, labelled by their maximum read id.
 */
#include <errno.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mp_oracle.h"

#define NB 1048576ull            /* 4^10 m-mer buckets */
#define REC_BYTES 4194344ull     /* sizeof(fileIndex) on LP64 */
#define REC_COUNTS_OFS 28ull
#define UMAX32 4294967295ull
#define BADV 0xBADBADBADull

static char g_err[512];
static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}
const char *mpo_last_error(void) { return g_err; }

/* ------------------------------------------------------------------ files */

typedef struct { char *data; uint64_t size; } mfile;

static int load_file(const char *path, mfile *m)
{
    FILE *f = fopen(path, "rb");
    if (!f) return fail(MPO_EIO, "cannot open %s", path);
    fseek(f, 0, SEEK_END);
    long long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    m->data = (char *)malloc((size_t)n + 16);
    if (!m->data) { fclose(f); return fail(MPO_ENOMEM, "out of memory reading %s", path); }
    if (n && fread(m->data, 1, (size_t)n, f) != (size_t)n) { fclose(f); return fail(MPO_EIO, "short read %s", path); }
    memset(m->data + n, 0, 16);
    m->size = (uint64_t)n;
    fclose(f);
    return 0;
}
static int load_files(int n, const char *const *paths, mfile *out)
{
    for (int i = 0; i < n; i++) {
        int rc = load_file(paths[i], &out[i]);
        if (rc) return rc;
    }
    return 0;
}
static void free_files(int n, mfile *f) { for (int i = 0; i < n; i++) free(f[i].data); }

/* index record header (genFastqIdx.c:11-18) */
typedef struct { uint64_t offset, offset2; uint8_t extra; uint32_t read_id; int32_t file_no; } rec_hdr;

static void put_hdr(unsigned char *r, const rec_hdr *h)
{
    memset(r, 0, REC_COUNTS_OFS);
    memcpy(r + 0, &h->offset, 8);
    memcpy(r + 8, &h->offset2, 8);
    r[16] = h->extra;
    memcpy(r + 20, &h->read_id, 4);
    memcpy(r + 24, &h->file_no, 4);
}
static void get_hdr(const unsigned char *r, rec_hdr *h)
{
    memcpy(&h->offset, r + 0, 8);
    memcpy(&h->offset2, r + 8, 8);
    h->extra = r[16];
    memcpy(&h->read_id, r + 20, 4);
    memcpy(&h->file_no, r + 24, 4);
}

static int check_kinds(int n_pe, int n_se, int n_il, int nfiles)
{
    if (n_pe != 0) return fail(MPO_EUNSUP, "two-file paired-end input is not supported");
    if (n_se < 0 || n_il < 0 || n_se + n_il != nfiles || nfiles < 1)
        return fail(MPO_EARG, "file counts do not match the file list");
    if (n_se > 0 && n_il > 0) return fail(MPO_EUNSUP, "mixing single-end and interleaved files is not supported");
    return 0;
}

/* ------------------------------------------------------- genFastqIdx */

/* genFastqIdx.c:28-53 with no two-file paired-end input */
static void file_index_of(uint64_t chunk, uint64_t per_chunk, const mfile *f, int *file_no, uint64_t *ofs)
{
    int cur = 0;
    uint64_t rem = per_chunk * chunk;
    while (rem >= f[cur].size) { rem -= f[cur].size; cur++; }
    *file_no = cur;
    *ofs = rem;
}

int mpo_fastq_index(int num_chunks, int n_pe, int n_se, int n_il, int nfiles, const char *const *files)
{
    int rc = check_kinds(n_pe, n_se, n_il, nfiles);
    if (rc) return rc;
    if (num_chunks <= 0) return fail(MPO_EARG, "numPartitions must be positive");
    mfile *f = (mfile *)calloc((size_t)nfiles, sizeof(mfile));
    if ((rc = load_files(nfiles, files, f))) { free_files(nfiles, f); free(f); return rc; }
    uint64_t total = 0;
    for (int i = 0; i < nfiles; i++) total += f[i].size;
    uint64_t per_chunk = total / (uint64_t)num_chunks;
    int max_read_size = 300, interleaved = 0;
    unsigned char *rec = (unsigned char *)calloc(1, REC_BYTES);
    char path[4096];
    snprintf(path, sizeof path, "%s.idx", files[0]);
    FILE *out = fopen(path, "wb");
    if (!out || !rec) { free(rec); free_files(nfiles, f); free(f); return fail(MPO_EIO, "cannot write %s", path); }
    rec_hdr h = {0, 0, 0, 0, 0};
    unsigned char buf[5000];
    for (int i = 0; i < num_chunks; i++) {
        file_index_of((uint64_t)i, per_chunk, f, &h.file_no, &h.offset);       /* :216 */
        if (h.file_no >= n_pe + n_se) interleaved = 1;                           /* :217 */
        if (f[h.file_no].size - h.offset < (uint64_t)max_read_size) {            /* :219-225 */
            if (h.file_no + 1 == nfiles) break;
            h.file_no++;
            h.offset = 0;
        }
        if (i == 0) {                                                            /* :228-249 */
            h.offset2 = 0; h.read_id = 0;
            put_hdr(rec, &h);
            fwrite(rec, 1, REC_BYTES, out);
            continue;
        }
        uint64_t avail = f[h.file_no].size - h.offset;
        size_t nread = (size_t)(avail < 3000 ? avail : 3000);                    /* :254 */
        memset(buf, 0, sizeof buf);
        memcpy(buf, f[h.file_no].data + h.offset, nread);
        if (nread <= (size_t)max_read_size) { rc = fail(MPO_EFMT, "chunk %d starts too close to the end of a file", i); goto done; }
        int flag = 0, k = 0, found = 0;
        size_t j;
#define B(x) ((x) < sizeof buf ? buf[(x)] : 0)
        for (j = 0; j < nread; j++) {                                            /* :258-302 */
            if (B(j) == '\n' && B(j + 1) == '+') {
                flag = 1;
                j += 2;
                while (j < sizeof buf && B(j) != '\n') j++;
                j++;
            }
            k = 0;
            if (flag && B(j) == '\n') {
                j++; k++;
                if (interleaved) {
                    char n1[200], n2[200];
                    size_t q;
                    for (q = j; q < sizeof buf && B(q) != '/' && B(q) != ' '; q++) if (q - j < 199) n1[q - j] = (char)B(q);
                    n1[(q - j) < 199 ? (q - j) : 199] = 0;
                    for (int l = 0; l < 4; l++) { while (q < sizeof buf && B(q) != '\n') q++; q++; }
                    size_t j2 = q;
                    while (q < sizeof buf && B(q) != ' ' && B(q) != '/') { if (q - j2 < 199) n2[q - j2] = (char)B(q); q++; }
                    n2[(q - j2) < 199 ? (q - j2) : 199] = 0;
                    if (q >= sizeof buf) { rc = fail(MPO_EFMT, "interleaved mate names not found near chunk %d", i); goto done; }
                    k = (int)q;
                    if (strcmp(n1, n2)) j = j2;
                }
                found = 1;
                break;
            }
        }
#undef B
        if (!found) { rc = fail(MPO_EFMT, "no record boundary within 3000 bytes of chunk %d", i); goto done; }
        if (2 * k + 30 < max_read_size) max_read_size = 2 * k + 30;             /* :303 */
        h.offset = h.offset + j;                                                 /* :305-307 */
        h.offset2 = 0;
        h.read_id = 0;
        put_hdr(rec, &h);
        fwrite(rec, 1, REC_BYTES, out);
    }
    h.file_no = nfiles - 1;                                                      /* :338-350 */
    h.offset = f[nfiles - 1].size;
    h.offset2 = 0;
    h.read_id = 0;
    put_hdr(rec, &h);
    fwrite(rec, 1, REC_BYTES, out);
    rc = 0;
done:
    fclose(out);
    free(rec);
    free_files(nfiles, f);
    free(f);
    return rc;
}

/* --------------------------------------------------------- FASTQ parse */

/* A record: header line, sequence line, '+' line, quality of the sequence's
 * length.  This is the layout getNextRead walks (genHistograms.c:60-80,
 * metapart.c:296-369) and getNextFullRead copies (metapart.c:211-294). */
typedef struct { uint64_t start, seq, end; uint32_t len; } rdesc;

typedef struct { char *buf; uint64_t n; rdesc *r; uint64_t nr; } chunk_view;

/* concatenates the chunk bytes [rec a, rec b) across files (loadChunk, metapart.c:371-500) */
static int chunk_bytes(const mfile *f, const rec_hdr *a, const rec_hdr *b, chunk_view *cv)
{
    uint64_t total = 0;
    for (int fn = a->file_no; fn <= b->file_no; fn++) {
        uint64_t s = (fn == a->file_no) ? a->offset : 0, e = (fn == b->file_no) ? b->offset : f[fn].size;
        if (e < s || e > f[fn].size) return fail(MPO_EFMT, "index record outside its file");
        total += e - s;
    }
    cv->buf = (char *)malloc((size_t)total + 16);
    if (!cv->buf) return fail(MPO_ENOMEM, "out of memory");
    uint64_t p = 0;
    for (int fn = a->file_no; fn <= b->file_no; fn++) {
        uint64_t s = (fn == a->file_no) ? a->offset : 0, e = (fn == b->file_no) ? b->offset : f[fn].size;
        memcpy(cv->buf + p, f[fn].data + s, (size_t)(e - s));
        p += e - s;
    }
    memset(cv->buf + total, 0, 16);
    cv->n = total;
    return 0;
}

static int parse_chunk(chunk_view *cv)
{
    const char *b = cv->buf;
    uint64_t n = cv->n, p = 0, cap = 1024, cnt = 0;
    rdesc *r = (rdesc *)malloc(cap * sizeof(rdesc));
    if (!r) return fail(MPO_ENOMEM, "out of memory");
    while (p < n) {
        rdesc d;
        d.start = p;
        while (p < n && b[p] != '\n') p++;
        if (p >= n) goto bad;
        p++;
        d.seq = p;
        while (p < n && b[p] != '\n') p++;
        if (p >= n) goto bad;
        d.len = (uint32_t)(p - d.seq);
        p++;
        while (p < n && b[p] != '\n') p++;
        if (p >= n) goto bad;
        p++;
        if (p + d.len >= n || b[p + d.len] != '\n') goto bad;
        p += d.len + 1;
        d.end = p;
        if (cnt == cap) {
            cap *= 2;
            rdesc *nr = (rdesc *)realloc(r, cap * sizeof(rdesc));
            if (!nr) { free(r); return fail(MPO_ENOMEM, "out of memory"); }
            r = nr;
        }
        r[cnt++] = d;
    }
    cv->r = r;
    cv->nr = cnt;
    return 0;
bad:
    free(r);
    return fail(MPO_EFMT, "malformed FASTQ record near byte %llu of a chunk", (unsigned long long)p);
}
static void chunk_free(chunk_view *cv) { free(cv->buf); free(cv->r); cv->buf = NULL; cv->r = NULL; }

/* ------------------------------------------------------------ k-mers */

static inline int fcode(unsigned char c) { static const int m[4] = {0, 1, 3, 2}; return m[(c & 6) >> 1]; }
static inline int rcode(unsigned char c) { static const int m[4] = {3, 2, 0, 1}; return m[(c & 6) >> 1]; }
static inline unsigned char cmpl(unsigned char c) { return (unsigned char)"TGAC   N"[(c >> 1) & 7]; }
static inline uint8_t adj_fwd(unsigned char p, unsigned char n) { return (uint8_t)((((unsigned)p << 2) & 0xF8) | ((n >> 1) & 7)); }
static inline uint8_t adj_rc(unsigned char p, unsigned char n) { return (uint8_t)((((unsigned)n << 2) & 0xF8) | ((p >> 1) & 7)); }

/* countMmers.c:83-217: canonical k-mer buckets of one read */
static uint64_t count_plain(const unsigned char *s, int L, int k, uint64_t *rh, uint32_t *cf)
{
    if (L <= k) return 0;
    int last = L - k, lastN = -1, sh = 2 * (k - 10);
    uint64_t mask = (1ull << (2 * k)) - 1, fwd = 0, rc = 0, n = 0;
    for (int j = 0; j < k; j++) {
        if (s[j] == 'N') lastN = j;
        rc |= (uint64_t)rcode(s[j]) << (2 * j);
        fwd = (fwd << 2) | (uint64_t)fcode(s[j]);
    }
    if (lastN == -1) { uint64_t b = (fwd < rc ? fwd : rc) >> sh; rh[b]++; cf[b]++; n++; }
    for (int i = 1; i <= last; i++) {
        unsigned char c = s[i + k - 1];
        rc = (rc >> 2) | ((uint64_t)rcode(c) << (2 * (k - 1)));
        fwd = ((fwd << 2) | (uint64_t)fcode(c)) & mask;
        if (c == 'N') lastN = i + k - 1;
        if (i > lastN) { uint64_t b = (fwd < rc ? fwd : rc) >> sh; rh[b]++; cf[b]++; n++; }
    }
    return n;
}

/* countMmers_3minimizers.c:83-271 */
static uint64_t count_min3(const unsigned char *s, int L, int k, uint64_t *rh, uint32_t *cf)
{
    if (L <= k) return 0;
    int last = L - k, lastN = -1, sh = 2 * (k - 10), win = last / 3, next_win = win;
    uint64_t mask = (1ull << (2 * k)) - 1, fwd = 0, rc = 0, n = 0, mn = 0, mb = 0;
    for (int j = 0; j < k; j++) {
        if (s[j] == 'N') lastN = j;
        rc |= (uint64_t)rcode(s[j]) << (2 * j);
        fwd = (fwd << 2) | (uint64_t)fcode(s[j]);
    }
    if (lastN == -1) { mn = fwd < rc ? fwd : rc; mb = mn >> sh; }
    for (int i = 1; i <= last; i++) {
        unsigned char c = s[i + k - 1];
        rc = (rc >> 2) | ((uint64_t)rcode(c) << (2 * (k - 1)));
        fwd = ((fwd << 2) | (uint64_t)fcode(c)) & mask;
        if (c == 'N') lastN = i + k - 1;
        if (i > lastN) {
            uint64_t v = fwd < rc ? fwd : rc, b = v >> sh;
            if (i > next_win) {
                if (mn != 0) { rh[mb]++; cf[mb]++; n++; }
                mn = v; mb = b;
                next_win += win;
                if (next_win + win > last) next_win = last;
            } else if (v < mn || mn == 0) { mn = v; mb = b; }
        }
    }
    if (mn != 0) { rh[mb]++; cf[mb]++; n++; }
    return n;
}

/* a sort tuple: the reference's 14-byte record unpacked (enumerateKmers.c:352-365) */
typedef struct { uint64_t kmer; uint32_t id; uint8_t adj; uint8_t pad[3]; } tup;

typedef struct { tup *t; uint64_t n, cap; } tvec;
static inline int tpush(tvec *v, uint64_t kmer, uint32_t id, uint8_t adj)
{
    if (v->n == v->cap) {
        uint64_t nc = v->cap ? v->cap * 2 : 4096;
        tup *nt = (tup *)realloc(v->t, nc * sizeof(tup));
        if (!nt) return -1;
        v->t = nt; v->cap = nc;
    }
    tup *x = &v->t[v->n++];
    x->kmer = kmer; x->id = id; x->adj = adj;
    x->pad[0] = x->pad[1] = x->pad[2] = 0;
    return 0;
}

/* enumerateKmers.c:127-371: in-range canonical k-mers of one read with adjacency */
static int enum_plain(const unsigned char *s, int L, int k, uint64_t lo, uint64_t hi, uint32_t id, tvec *out)
{
    if (L <= k) return 0;
    if (out->cap - out->n < (uint64_t)(L - k + 1)) {  /* room for every position, so tpush never grows */
        uint64_t nc = out->cap ? out->cap : 4096;
        while (nc - out->n < (uint64_t)(L - k + 1)) nc *= 2;
        tup *nt = (tup *)realloc(out->t, nc * sizeof(tup));
        if (!nt) return -1;
        out->t = nt;
        out->cap = nc;
    }
    int last = L - k, lastN = -1, sh = 2 * (k - 10);
    uint64_t mask = (1ull << (2 * k)) - 1, fwd = 0, rc = 0;
    unsigned char prev = 'N', next = s[k];
    for (int j = 0; j < k; j++) {
        if (s[j] == 'N') lastN = j;
        rc |= (uint64_t)rcode(s[j]) << (2 * j);
        fwd = (fwd << 2) | (uint64_t)fcode(s[j]);
    }
    for (int i = 0; i <= last; i++) {
        if (i > 0) {
            prev = s[i - 1];
            next = (i == last) ? 'N' : s[i + k];
            unsigned char c = s[i + k - 1];
            rc = (rc >> 2) | ((uint64_t)rcode(c) << (2 * (k - 1)));
            fwd = ((fwd << 2) | (uint64_t)fcode(c)) & mask;
            if (c == 'N') lastN = i + k - 1;
            if (!(i > lastN)) continue;
        } else if (lastN != -1) {
            continue;
        }
        /* written in place and kept when in range, without branches on the (unpredictable) orientation and
           range tests: the room is reserved above */
        const int f = fwd < rc;
        const uint64_t canon = f ? fwd : rc, b = canon >> sh;
        const uint8_t a_f = adj_fwd(prev, next), a_r = adj_rc(cmpl(prev), cmpl(next));
        tup *x = &out->t[out->n];
        x->kmer = canon;
        x->id = id;
        x->adj = f ? a_f : a_r;
        x->pad[0] = x->pad[1] = x->pad[2] = 0;
        out->n += (b >= lo) & (b < hi);
    }
    return 0;
}

/* enumerateKmers_3minimizers.c:129-470 */
static int enum_min3(const unsigned char *s, int L, int k, uint64_t lo, uint64_t hi, uint32_t id, tvec *out)
{
    if (L <= k) return 0;
    int last = L - k, lastN = -1, sh = 2 * (k - 10), win, next_win;
    uint64_t mask = (1ull << (2 * k)) - 1, fwd = 0, rc = 0, mn = 0;
    unsigned char prev = 'N', next = s[k], mprev = 0, mnext = 0;
    for (int j = 0; j < k; j++) {
        if (s[j] == 'N') lastN = j;
        rc |= (uint64_t)rcode(s[j]) << (2 * j);
        fwd = (fwd << 2) | (uint64_t)fcode(s[j]);
    }
    if (lastN == -1) {                                                  /* :201-261 */
        if (fwd < rc) {
            uint64_t b = fwd >> sh;
            if (b >= lo && b < hi) { mn = fwd; mprev = prev; mnext = next; }
        } else {
            uint64_t b = rc >> sh;
            if (b >= lo && b < hi) { mn = rc; mprev = cmpl(prev); mnext = cmpl(next); }
        }
    }
    win = last / 3;
    next_win = win;
    for (int i = 1; i <= last; i++) {                                   /* :267-415 */
        prev = s[i - 1];
        next = (i == last) ? 'N' : s[i + k];
        unsigned char c = s[i + k - 1];
        rc = (rc >> 2) | ((uint64_t)rcode(c) << (2 * (k - 1)));
        fwd = ((fwd << 2) | (uint64_t)fcode(c)) & mask;
        if (c == 'N') lastN = i + k - 1;
        if (!(i > lastN)) continue;
        int is_fwd = fwd < rc;
        uint64_t v = is_fwd ? fwd : rc, b = v >> sh;
        if (!(b >= lo && b < hi)) continue;
        unsigned char p = is_fwd ? prev : cmpl(prev), nx = is_fwd ? next : cmpl(next);
        if (i > next_win) {
            if (mn != 0) {
                uint8_t a = is_fwd ? adj_fwd(mprev, mnext) : adj_rc(mprev, mnext);
                if (tpush(out, mn, id, a)) return -1;
            }
            mn = v; mprev = p; mnext = nx;
            next_win += win;
            if (next_win + win > last) next_win = last;
        } else if (v < mn || mn == 0) {
            mn = v; mprev = p; mnext = nx;
        }
    }
    if (mn != 0 && tpush(out, mn, id, adj_rc(mprev, mnext))) return -1;  /* :418-426 */
    return 0;
}

/* ---------------------------------------------------- genHistograms */

static void hist_name(char *out, size_t n, const char *fq, const char *what, int min3, int k)
{
    snprintf(out, n, "%s.%s%s%d", fq, what, min3 ? "_3min" : "", k);
}

static int read_index(const char *path, unsigned char **recs, uint64_t *nrec)
{
    mfile m;
    int rc = load_file(path, &m);
    if (rc) return rc;
    if (m.size < 2 * REC_BYTES || m.size % REC_BYTES) { free(m.data); return fail(MPO_EFMT, "%s is not an index file", path); }
    *recs = (unsigned char *)m.data;
    *nrec = m.size / REC_BYTES;
    return 0;
}

int mpo_gen_histograms(int k, int min3, int n_pe, int n_se, int n_il, int nfiles, const char *const *files)
{
    int rc = check_kinds(n_pe, n_se, n_il, nfiles);
    if (rc) return rc;
    if (k < 11 || k > 31) return fail(MPO_EARG, "k must be in [11, 31]");
    char path[4096];
    snprintf(path, sizeof path, "%s.idx", files[0]);
    unsigned char *recs = NULL;
    uint64_t nrec = 0;
    if ((rc = read_index(path, &recs, &nrec))) return rc;
    uint64_t nchunks = nrec - 1;
    mfile *f = (mfile *)calloc((size_t)nfiles, sizeof(mfile));
    if ((rc = load_files(nfiles, files, f))) { free_files(nfiles, f); free(f); free(recs); return rc; }
    uint64_t *reads = (uint64_t *)calloc(nchunks, sizeof(uint64_t));
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    uint64_t *rh = (uint64_t *)calloc((size_t)nth * NB, sizeof(uint64_t));
    if (!reads || !rh) { rc = fail(MPO_ENOMEM, "out of memory"); goto out; }
    int err = 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (uint64_t c = 0; c < nchunks; c++) {                           /* genHistograms.c:200-265 */
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        rec_hdr a, b;
        get_hdr(recs + c * REC_BYTES, &a);
        get_hdr(recs + (c + 1) * REC_BYTES, &b);
        uint32_t *cf = (uint32_t *)(recs + c * REC_BYTES + REC_COUNTS_OFS);
        memset(cf, 0, (NB + 2) * sizeof(uint32_t));
        chunk_view cv = {0};
        int lrc = chunk_bytes(f, &a, &b, &cv);
        if (!lrc) lrc = parse_chunk(&cv);
        if (lrc) {
#pragma omp critical
            err = lrc;
            chunk_free(&cv);
            continue;
        }
        for (uint64_t r = 0; r < cv.nr; r++) {
            const unsigned char *s = (const unsigned char *)cv.buf + cv.r[r].seq;
            if (min3) count_min3(s, (int)cv.r[r].len, k, rh + (size_t)t * NB, cf);
            else count_plain(s, (int)cv.r[r].len, k, rh + (size_t)t * NB, cf);
        }
        reads[c] = cv.nr;
        chunk_free(&cv);
    }
    if (err) { rc = err; goto out; }
    /* read ids: genHistograms.c:280-291 (record 0 keeps the index's values) */
    uint64_t acc = 0;
    for (uint64_t i = 1; i <= nchunks; i++) {
        acc += reads[i - 1];
        rec_hdr h;
        get_hdr(recs + i * REC_BYTES, &h);
        h.read_id = (uint32_t)(acc % UMAX32);
        if (acc / UMAX32 >= 256) { rc = fail(MPO_EUNSUP, "too many reads"); goto out; }
        h.extra = (uint8_t)(acc / UMAX32);
        memcpy(recs + i * REC_BYTES + 16, &h.extra, 1);
        memcpy(recs + i * REC_BYTES + 20, &h.read_id, 4);
    }
    char out_path[4096];
    hist_name(out_path, sizeof out_path, files[0], "KmerIdx", min3, k);
    FILE *fo = fopen(out_path, "wb");
    if (!fo) { rc = fail(MPO_EIO, "cannot write %s", out_path); goto out; }
    fwrite(recs, 1, nrec * REC_BYTES, fo);
    fclose(fo);
    /* histogram: exclusive prefix over buckets (genHistograms.c:302-343) */
    uint64_t *h = (uint64_t *)calloc(NB + 1, sizeof(uint64_t));
    if (!h) { rc = fail(MPO_ENOMEM, "out of memory"); goto out; }
    for (uint64_t b = 1; b <= NB; b++) {
        uint64_t cnt = 0;
        for (int t = 0; t < nth; t++) cnt += rh[(size_t)t * NB + b - 1];
        h[b] = h[b - 1] + cnt;
    }
    hist_name(out_path, sizeof out_path, files[0], "kmerHist", min3, k);
    fo = fopen(out_path, "wb");
    if (!fo) { free(h); rc = fail(MPO_EIO, "cannot write %s", out_path); goto out; }
    fwrite(h, sizeof(uint64_t), NB + 1, fo);
    fclose(fo);
    free(h);
    rc = 0;
out:
    free(rh);
    free(reads);
    free(recs);
    free_files(nfiles, f);
    free(f);
    return rc;
}

/* ------------------------------------------------------------ metapart */

static uint64_t *g_parent;   /* parent array: value or BADV (unionfind.h 5-byte encoding, unpacked) */
static uint32_t *g_sizes;    /* compSizes */
static uint8_t *g_filtered;  /* filteredReads */
static uint64_t g_nreads;

/* unionfind.h:19-55: path halving that stops at BAD */
static uint64_t find_root(uint64_t e)
{
    uint64_t p = g_parent[e];
    if (p == BADV) return e;
    while (p != e) {
        if (p == BADV) break;
        uint64_t pp = g_parent[p];
        if (p != BADV && pp != BADV) { g_parent[e] = pp; p = pp; }
        if (p != BADV) e = p; else break;
        p = g_parent[e];
    }
    return e;
}

/* printStats, metapart.c:3227-3308 */
static void print_stats(void)
{
    for (uint64_t r = 0; r < g_nreads; r++) {
        uint64_t tp = g_parent[r];
        if (tp != BADV) {
            tp = find_root(r);
            g_parent[r] = tp;
        }
        if (tp != r && tp != BADV) {
            g_sizes[r] = 0;
            g_sizes[tp]++;
        }
    }
}

/* unionFindPeReads, metapart.c:2801-2867 (unionOp: unionfind.h:58-85) */
static void pe_union(uint32_t upto)
{
    for (uint64_t i = 0; i < g_nreads; i += 2) {
        uint64_t a = i, b = i + 1;
        if (g_parent[a] == BADV) g_parent[a] = a;
        if (g_parent[b] == BADV) g_parent[b] = b;
        uint64_t pa = find_root(a), pb = find_root(b);
        if (g_sizes[pa] <= upto || g_sizes[pb] <= upto) {
            uint64_t u = find_root(a), v = find_root(b);
            if (u != v) {
                uint64_t hi = u > v ? u : v, lo = u > v ? v : u;
                g_parent[lo] = hi;
                g_sizes[hi] += g_sizes[lo];
                g_sizes[lo] = 0;
            }
        }
    }
}

static void dump(const char *name, const void *buf, size_t bytes)
{
    const char *dir = getenv("MP_DUMP_DIR");
    if (!dir) return;
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) return;
    if (bytes) fwrite(buf, 1, bytes, f);
    fclose(f);
}
static void dump_tuples(const char *name, const tup *t, uint64_t n)
{
    if (!getenv("MP_DUMP_DIR")) return;
    const char *tu = getenv("MP_DUMP_TUPLES");  /* "0": the per-read dumps only (large inputs) */
    if (tu && strcmp(tu, "0") == 0) return;
    unsigned char *b = (unsigned char *)malloc(n * 14 + 1);
    for (uint64_t i = 0; i < n; i++) {
        unsigned char *o = b + i * 14;
        uint16_t w4 = (uint16_t)((uint16_t)((t[i].id / UMAX32) << 8) | t[i].adj);
        uint32_t rem = (uint32_t)(t[i].id % UMAX32);
        memcpy(o, &t[i].kmer, 8);
        memcpy(o + 8, &w4, 2);
        memcpy(o + 10, &rem, 4);
    }
    dump(name, b, n * 14);
    free(b);
}
static void dump_state(const char *pname, const char *sname)
{
    if (!getenv("MP_DUMP_DIR")) return;
    unsigned char *b = (unsigned char *)malloc(g_nreads * 5 + 1);
    for (uint64_t i = 0; i < g_nreads; i++) {
        uint32_t rem = (uint32_t)(g_parent[i] % UMAX32);
        b[i * 5] = (uint8_t)(g_parent[i] / UMAX32);
        memcpy(b + i * 5 + 1, &rem, 4);
    }
    dump(pname, b, g_nreads * 5);
    free(b);
    dump(sname, g_sizes, g_nreads * 4);
}

/* metapart.c:3720-3791 (one rank) */
static int plan_ranges(const uint64_t *hist, int scans, int T, uint64_t *scanR, uint64_t *thrR)
{
    uint64_t total = hist[NB];
    if (total == 0) return fail(MPO_EUNSUP, "the histogram holds no k-mers");
    uint64_t avg = total / (uint64_t)scans + (total % (uint64_t)scans ? 1 : 0);
    uint64_t cr = 1, i;
    scanR[0] = 0;
    for (i = 0; i < NB; i++)
        if (hist[i] >= avg * cr) { if (cr <= (uint64_t)scans) scanR[cr] = i; cr++; }
    if (cr == (uint64_t)scans) scanR[cr] = i;
    /* processKmerRanges equals scanKmerRanges at one rank (:3750-3770) */
    uint64_t avgT = avg / (uint64_t)T;
    cr = 1;
    thrR[0] = 0;
    for (i = 0; i < NB; i++)
        if (hist[i] >= cr * avgT) {
            if (cr <= (uint64_t)scans * T) thrR[cr] = (cr % (uint64_t)T == 0) ? scanR[cr / T] : i;
            cr++;
        }
    if (cr == (uint64_t)scans * T) thrR[cr] = i;
    return 0;
}

/* range partition bin of a bucket (metapart.c:2019-2022) */
/* radixPass (metapart.c:1494-1598) over passOrder 5..13 (:2169-2195): adj byte, then k-mer bytes 0..7.
   A digit that is the same in every tuple of the bin moves nothing in a stable pass, so it is skipped;
   the passes alternate between the two buffers and the result is copied back once. */
static void sort_bin(tup *a, tup *tmp, uint64_t n)
{
    uint64_t cnt[9][257];
    memset(cnt, 0, sizeof cnt);
    for (uint64_t i = 0; i < n; i++) {
        cnt[0][a[i].adj + 1]++;
        const uint64_t km = a[i].kmer;
        for (int b = 0; b < 8; b++) cnt[b + 1][((km >> (8 * b)) & 0xFF) + 1]++;
    }
    tup *src = a, *dst = tmp;
    for (int pass = 0; pass < 9; pass++) {
        int constant = 0;
        for (int d = 1; d <= 256; d++)
            if (cnt[pass][d] == n) constant = 1;
        if (constant) continue;
        uint64_t *c = cnt[pass];
        for (int d = 1; d <= 256; d++) c[d] += c[d - 1];
        for (uint64_t i = 0; i < n; i++) {
            unsigned d = pass == 0 ? src[i].adj : (unsigned)((src[i].kmer >> (8 * (pass - 1))) & 0xFF);
            dst[c[d]++] = src[i];
        }
        tup *x = src; src = dst; dst = x;
    }
    if (src != a) memcpy(a, src, n * sizeof(tup));
}

/* markMischiefKmers body for one thread range (metapart.c:2276-2468) */
static void mischief(tup *t, uint64_t n)
{
    if (n == 0) return;
    uint64_t cur = t[0].kmer, cur_ofs = 0;
    int before[8] = {0}, after[8] = {0}, deg = 0;
    for (uint64_t j = 0; j < n; j++) {
        uint64_t nk = t[j].kmer;
        if (cur != nk) {
            int nin = 0, nout = 0, mxi = 0, mxo = 0, cmi = 0, cmo = 0, smi = 0, smo = 0;
            for (int q = 0; q < 7; q++) {
                if (before[q]) {
                    if (before[q] > cmi) { smi = cmi; cmi = before[q]; mxi = q; }
                    else if (before[q] > smi) { smi = before[q]; }
                    nin++;
                }
                if (after[q]) {
                    if (after[q] > cmo) { smo = cmo; cmo = after[q]; mxo = q; }
                    else if (after[q] > smo) { smo = after[q]; }
                    nout++;
                }
            }
            if (nin > 1 || nout > 1) {
                float s_in = (float)smi / (float)deg, s_out = (float)smo / (float)deg;
                for (uint64_t q = cur_ofs; q < j; q++) {
                    unsigned bi = t[q].adj & 7, ai = (t[q].adj >> 3) & 7;
                    if (nin > 1 && nout > 1) { t[q].kmer = 0; continue; }
                    int bad = (nin > 1 && bi != (unsigned)mxi) || (nout > 1 && ai != (unsigned)mxo);
                    if (!bad) bad = ((double)s_in > 0.2) || ((double)s_out > 0.2);
                    if (bad) { g_parent[t[q].id] = BADV; g_filtered[t[q].id] = 1; }
                }
            }
            cur = nk;
            cur_ofs = j;
            deg = 0;
            for (int q = 0; q < 8; q++) before[q] = after[q] = 0;
        }
        before[t[j].adj & 7]++;
        after[(t[j].adj >> 3) & 7]++;
        deg++;
    }
}

/* unionFindPar2 body for one thread range (metapart.c:2537-2727), applied sequentially.  The initial
   anchor (the scan's first read) may be BAD: findRoot returns it as its own root and the hooks go on as
   for any read.  Returns 1 when it united that BAD read (the caller checks the replay's assertion). */
static int range_unions(const tup *t, uint64_t n, uint64_t init_kmer, uint64_t init_min)
{
    uint64_t cur = init_kmer, mn = init_min;
    int bad_anchor = 0;
    for (uint64_t i = 0; i < n; i++) {
        uint64_t id = t[i].id;
        if (g_parent[id] == BADV) continue;
        if (t[i].kmer == 0) continue;
        if (t[i].kmer != cur) { cur = t[i].kmer; mn = id; continue; }
        if (mn == init_min && g_parent[mn] == BADV) bad_anchor = 1;
        uint64_t pu = mn, pv = id;
        if (pu != pv) { pu = find_root(pu); pv = find_root(pv); }
        if (pu != pv) {
            if (pu > pv) g_parent[pv] = pu; else g_parent[pu] = pv;
        }
    }
    return bad_anchor;
}

typedef struct { FILE **fp; int T; } outset;

int mpo_metapart(const char *out_prefix, uint64_t fastq_buffer_size, int k, int num_scans, int num_threads,
                 int min3, int n_pe, int n_se, int n_il, int nfiles, const char *const *files)
{
    int rc = check_kinds(n_pe, n_se, n_il, nfiles);
    if (rc) return rc;
    if (k < 11 || k > 31) return fail(MPO_EARG, "k must be in [11, 31]");
    if (num_scans < 1 || num_threads < 1 || num_threads > 256) return fail(MPO_EARG, "bad numScans/numThreads");
    if (min3 && num_scans != 1) return fail(MPO_EUNSUP, "the 3-minimizer variant needs numScans == 1");
    const int T = num_threads, S = num_scans;
    char path[4096];
    unsigned char *recs = NULL;
    uint64_t nrec = 0;
    hist_name(path, sizeof path, files[0], "KmerIdx", min3, k);
    if ((rc = read_index(path, &recs, &nrec))) return rc;
    uint64_t nchunks = nrec - 1;
    if (nchunks % (uint64_t)T) { free(recs); return fail(MPO_EARG, "numThreads must divide the chunk count"); }
    uint64_t per_thread = nchunks / (uint64_t)T;
    rec_hdr *hd = (rec_hdr *)malloc(nrec * sizeof(rec_hdr));
    for (uint64_t i = 0; i < nrec; i++) get_hdr(recs + i * REC_BYTES, &hd[i]);
    free(recs);
    g_nreads = (uint64_t)hd[nchunks].extra * UMAX32 + hd[nchunks].read_id;
    if (g_nreads & 1) { free(hd); return fail(MPO_EUNSUP, "the mate union needs an even read count"); }
    if (g_nreads >= UMAX32) { free(hd); return fail(MPO_EUNSUP, "too many reads"); }
    uint64_t *hist = (uint64_t *)malloc((NB + 1) * sizeof(uint64_t));
    hist_name(path, sizeof path, files[0], "kmerHist", min3, k);
    FILE *fh = fopen(path, "rb");
    if (!fh || fread(hist, sizeof(uint64_t), NB + 1, fh) != NB + 1) {
        if (fh) fclose(fh);
        free(hd); free(hist);
        return fail(MPO_EIO, "cannot read %s", path);
    }
    fclose(fh);
    uint64_t *scanR = (uint64_t *)calloc((size_t)S + 1, sizeof(uint64_t));
    uint64_t *thrR = (uint64_t *)calloc((size_t)S * T + 1, sizeof(uint64_t));
    mfile *f = (mfile *)calloc((size_t)nfiles, sizeof(mfile));
    tvec *per = (tvec *)calloc((size_t)T, sizeof(tvec));
    chunk_view *cvs = (chunk_view *)calloc(nchunks, sizeof(chunk_view));
    tup *arr = NULL, *tmp = NULL;
    uint64_t arr_cap = 0;
    g_parent = NULL; g_sizes = NULL; g_filtered = NULL;
    if ((rc = plan_ranges(hist, S, T, scanR, thrR))) goto out;
    if ((rc = load_files(nfiles, files, f))) goto out;
    {   /* the chunks in parallel; the first failing chunk (in chunk order) is redone alone for its message */
        int *crc = (int *)calloc(nchunks, sizeof(int));
        if (!crc) { rc = fail(MPO_ENOMEM, "out of memory"); goto out; }
#pragma omp parallel for schedule(dynamic, 1)
        for (uint64_t c = 0; c < nchunks; c++) {
            chunk_view cv = {0};
            int r = chunk_bytes(f, &hd[c], &hd[c + 1], &cv);
            if (!r && cv.n >= fastq_buffer_size) r = MPO_EARG;
            if (!r) r = parse_chunk(&cv);
            crc[c] = r;
            cvs[c] = cv;
        }
        for (uint64_t c = 0; c < nchunks && !rc; c++) {
            if (!crc[c]) continue;
            chunk_free(&cvs[c]);
            if ((rc = chunk_bytes(f, &hd[c], &hd[c + 1], &cvs[c]))) break;
            if (cvs[c].n >= fastq_buffer_size) { rc = fail(MPO_EARG, "fastqBufferSize is smaller than a chunk"); break; }
            rc = parse_chunk(&cvs[c]);
            if (!rc) rc = fail(crc[c], "chunk %llu failed", (unsigned long long)c);
        }
        free(crc);
        if (rc) goto out;
    }
    {
        uint64_t nread_seen = 0;
        for (uint64_t c = 0; c < nchunks; c++) nread_seen += cvs[c].nr;
        if (nread_seen != g_nreads) { rc = fail(MPO_EFMT, "index read count does not match the FASTQ"); goto out; }
        if (n_il) for (uint64_t c = 0; c < nchunks; c++)
            if (cvs[c].nr & 1) { rc = fail(MPO_EFMT, "interleaved chunk with an odd record count"); goto out; }
    }
    const int sh = 2 * (k - 10);
    for (int s = 0; s < S; s++) {
        uint64_t lo = scanR[s], hi = scanR[s + 1];
        /* generateKmersInScan (metapart.c:1192-1476): threads in order = enumeration order */
        int err = 0;
#pragma omp parallel for schedule(dynamic, 1)
        for (int t = 0; t < T; t++) {
            per[t].n = 0;
            for (uint64_t c = (uint64_t)t * per_thread; c < (uint64_t)(t + 1) * per_thread; c++) {
                uint64_t rid = (uint64_t)hd[c].extra * UMAX32 + hd[c].read_id;
                for (uint64_t r = 0; r < cvs[c].nr; r++, rid++) {
                    const unsigned char *sq = (const unsigned char *)cvs[c].buf + cvs[c].r[r].seq;
                    uint64_t id = g_parent ? find_root(rid) : rid;          /* SCAN_OPT :543-568 */
                    const uint64_t before = per[t].n;
                    int e = min3 ? enum_min3(sq, (int)cvs[c].r[r].len, k, lo, hi, (uint32_t)id, &per[t])
                                 : enum_plain(sq, (int)cvs[c].r[r].len, k, lo, hi, (uint32_t)id, &per[t]);
                    if (e) err = 1;
                    /* the reference counts a read's tuples in a uint8_t (enumerateKmers.c:152, 212, 343):
                       256 or more in one scan overlap the next read's */
                    if (per[t].n - before > 255) err = 2;
                }
            }
        }
        if (err == 2) { rc = fail(MPO_EUNSUP, "a read has 256 or more k-mers in one scan"); goto out; }
        if (err) { rc = fail(MPO_ENOMEM, "out of memory enumerating"); goto out; }
        uint64_t n = 0;
        for (int t = 0; t < T; t++) n += per[t].n;
        if (n + 1 > arr_cap) {  /* the scan arrays, kept from scan to scan */
            free(arr); free(tmp);
            arr_cap = n + 1;
            arr = (tup *)malloc(arr_cap * sizeof(tup));
            tmp = (tup *)malloc(arr_cap * sizeof(tup));
            if (!arr || !tmp) { rc = fail(MPO_ENOMEM, "out of memory"); goto out; }
        }
        {
            uint64_t at[257];
            at[0] = 0;
            for (int t = 0; t < T; t++) at[t + 1] = at[t] + per[t].n;
#pragma omp parallel for schedule(dynamic, 1)
            for (int t = 0; t < T; t++) memcpy(arr + at[t], per[t].t, per[t].n * sizeof(tup));
        }
        char name[64];
        snprintf(name, sizeof name, "scan%d_enum.bin", s);
        dump_tuples(name, arr, n);
        if (!g_parent) {                                                     /* :3933-3954 */
            g_parent = (uint64_t *)malloc(g_nreads * sizeof(uint64_t));
            g_sizes = (uint32_t *)malloc(g_nreads * sizeof(uint32_t));
            g_filtered = (uint8_t *)calloc(g_nreads, 1);
            if (!g_parent || !g_sizes || !g_filtered) { rc = fail(MPO_ENOMEM, "out of memory"); goto out; }
            for (uint64_t r = 0; r < g_nreads; r++) { g_parent[r] = r; g_sizes[r] = 1; }
        }
        /* sortKmerList: stable range partition into thread bins, then LSD per bin */
        const uint64_t *ltr = thrR + (size_t)s * T;
        uint64_t bcount[257] = {0}, refcount[257] = {0};
        /* the range partition's bin of a tuple (metapart.c:2019-2022): walking the range starts from the
           first, the bin before the first start above the bucket; that start is the first running maximum
           of the starts above the bucket, so a binary search over the running maxima finds it */
        uint64_t M[258];
        M[0] = ltr[0];
        for (int t = 1; t <= T; t++) M[t] = M[t - 1] > ltr[t] ? M[t - 1] : ltr[t];
        uint16_t *bin = (uint16_t *)malloc((n + 1) * sizeof(uint16_t));
        if (!bin) { rc = fail(MPO_ENOMEM, "out of memory"); goto out; }
        int bad_bin = 0;
#pragma omp parallel for schedule(static)
        for (uint64_t i = 0; i < n; i++) {
            const uint64_t b = arr[i].kmer >> sh;
            int l = 0, h = T + 1;  /* first t in [0, T] with M[t] > b (T + 1: none) */
            while (l < h) { int m = (l + h) >> 1; if (M[m] > b) h = m; else l = m + 1; }
            const int cb = l - 1;
            if (cb < 0 || cb >= T) bad_bin = 1;
            bin[i] = (uint16_t)(cb < 0 ? 0 : cb);
        }
        if (bad_bin) { free(bin); rc = fail(MPO_EUNSUP, "thread k-mer ranges do not cover a bucket"); goto out; }
        for (uint64_t i = 0; i < n; i++) bcount[bin[i] + 1]++;
        /* the reference sizes bins from bucket counts over [ltr[t], ltr[t+1]) (:1810-1850) */
        for (int t = 0; t < T; t++) {
            uint64_t a = ltr[t], b = ltr[t + 1];
            refcount[t + 1] = (b > a) ? hist[b] - hist[a] : 0;
            if (refcount[t + 1] != bcount[t + 1]) {
                free(bin);
                rc = fail(MPO_EUNSUP, "thread k-mer ranges are not monotone over populated buckets");
                goto out;
            }
        }
        for (int t = 0; t < T; t++) bcount[t + 1] += bcount[t];
        {  /* stable scatter into the bins: the input in NP parts, each part's tuples of a bin after the earlier
              parts' (counts per part and bin, then every part scatters on its own) */
            enum { NP = 64 };
            static uint64_t pc[NP][257];
            memset(pc, 0, sizeof pc);
#pragma omp parallel for schedule(static)
            for (int q = 0; q < NP; q++)
                for (uint64_t i = n * q / NP; i < n * (q + 1) / NP; i++) pc[q][bin[i]]++;
            for (int t = 0; t < T; t++) {
                uint64_t at = bcount[t];
                for (int q = 0; q < NP; q++) {
                    const uint64_t c = pc[q][t];
                    pc[q][t] = at;
                    at += c;
                }
            }
#pragma omp parallel for schedule(static)
            for (int q = 0; q < NP; q++)
                for (uint64_t i = n * q / NP; i < n * (q + 1) / NP; i++) tmp[pc[q][bin[i]]++] = arr[i];
            memcpy(arr, tmp, n * sizeof(tup));
        }
        free(bin);
#pragma omp parallel for schedule(dynamic, 1)
        for (int t = 0; t < T; t++) sort_bin(arr + bcount[t], tmp + bcount[t], bcount[t + 1] - bcount[t]);
        snprintf(name, sizeof name, "scan%d_sorted.bin", s);
        dump_tuples(name, arr, n);
        /* markMischiefKmers (:2270-2519) */
#pragma omp parallel for schedule(dynamic, 1)
        for (int t = 0; t < T; t++) mischief(arr + bcount[t], bcount[t + 1] - bcount[t]);
        for (uint64_t r = 0; r < g_nreads; r++)
            if (g_parent[r] != BADV && g_filtered[r]) g_parent[r] = BADV;
        snprintf(name, sizeof name, "scan%d_filtered.bin", s);
        dump_tuples(name, arr, n);
        snprintf(name, sizeof name, "scan%d_bad.bin", s);
        dump(name, g_filtered, g_nreads);
        /* unionFindPar2 + unionFind (:2520-2800) */
        if (n) {
            uint64_t init_kmer = arr[n - 1].kmer, init_min = arr[0].id;
            int bad_anchor = 0;
            for (int t = 0; t < T; t++)
                bad_anchor |= range_unions(arr + bcount[t], bcount[t + 1] - bcount[t], init_kmer, init_min);
            /* the replay (unionFind, metapart.c:2772) asserts that no edge's read has a BAD parent: a BAD first
               read that no union hooked below a larger root stops the reference here */
            if (bad_anchor && g_parent[init_min] == BADV) {
                rc = fail(MPO_EUNSUP, "scan %d: the first read (%llu) is BAD and its run's roots are all smaller; the "
                          "reference's edge replay asserts (metapart.c:2772)", s, (unsigned long long)init_min);
                goto out;
            }
        }
        print_stats();
        snprintf(name, sizeof name, "stats%d_parent.bin", s);
        char name2[64];
        snprintf(name2, sizeof name2, "stats%d_sizes.bin", s);
        dump_state(name, name2);
    }
    /* final steps, metapart.c:4010-4053 */
    for (uint64_t r = 0; r < g_nreads; r++) g_sizes[r] = 1;
    print_stats();
    {
        char a[64], b[64];
        snprintf(a, sizeof a, "stats%d_parent.bin", S);
        snprintf(b, sizeof b, "stats%d_sizes.bin", S);
        dump_state(a, b);
    }
    pe_union(1000);
    dump_state("pe_parent.bin", "pe_sizes.bin");
    for (uint64_t r = 0; r < g_nreads; r++) g_sizes[r] = 1;
    print_stats();
    {
        char a[64], b[64];
        snprintf(a, sizeof a, "stats%d_parent.bin", S + 1);
        snprintf(b, sizeof b, "stats%d_sizes.bin", S + 1);
        dump_state(a, b);
    }
    uint64_t parts[17] = {0};
    {
        const int NP = 16;
        uint64_t per = g_nreads / NP, total = 0, ci = 0;
        parts[NP] = g_nreads;
        for (int i = 1; i < NP; i++) {
            while (ci < g_nreads && total < (uint64_t)i * per) {
                if (g_parent[ci] == ci) total += g_sizes[ci];
                ci++;
            }
            parts[i] = ci;
        }
    }
    /* writeOutput3 (:956-1066) */
    {
        FILE **fp = (FILE **)calloc((size_t)16 * T, sizeof(FILE *));
        for (int j = 0; j < 16 * T; j++) {
            int pid = j / T, tid = j % T;
            snprintf(path, sizeof path, "%s/Rank0/FromTid%d_ToRank%d.paired.fastq", out_prefix, tid, pid);
            fp[j] = fopen(path, "wb");
            if (!fp[j]) {
                for (int q = 0; q < j; q++) fclose(fp[q]);
                free(fp);
                rc = fail(MPO_EIO, "cannot write %s", path);
                goto out;
            }
        }
        /* every thread writes only its own files (FromTid<t>_*), as the reference's threads do */
#pragma omp parallel for schedule(dynamic, 1)
        for (int t = 0; t < T; t++) {
            for (uint64_t c = (uint64_t)t * per_thread; c < (uint64_t)(t + 1) * per_thread; c++) {
                uint64_t rid = (uint64_t)hd[c].extra * UMAX32 + hd[c].read_id;
                for (uint64_t r = 0; r < cvs[c].nr; r++) {
                    uint64_t pu = g_parent[rid];
                    int cu = 0;
                    while (cu < 16 && !(pu < parts[cu + 1])) cu++;
                    const char *b1 = cvs[c].buf + cvs[c].r[r].start;
                    size_t l1 = (size_t)(cvs[c].r[r].end - cvs[c].r[r].start);
                    if (n_il) {
                        const char *b2 = cvs[c].buf + cvs[c].r[r + 1].start;
                        size_t l2 = (size_t)(cvs[c].r[r + 1].end - cvs[c].r[r + 1].start);
                        uint64_t mate = (rid % 2 == 0) ? rid + 1 : rid - 1;
                        uint64_t pv = g_parent[mate];
                        int cv2 = 0;
                        while (cv2 < 16 && !(pv < parts[cv2 + 1])) cv2++;
                        fwrite(b1, 1, l1, fp[cu * T + t]);
                        fwrite(b2, 1, l2, fp[cu * T + t]);
                        if (pu != pv) {
                            fwrite(b1, 1, l1, fp[cv2 * T + t]);
                            fwrite(b2, 1, l2, fp[cv2 * T + t]);
                        }
                        r++;
                        rid += 2;
                    } else {
                        fwrite(b1, 1, l1, fp[cu * T + t]);
                        rid++;
                    }
                }
            }
        }
        for (int j = 0; j < 16 * T; j++) fclose(fp[j]);
        free(fp);
    }
    rc = 0;
out:
    if (cvs) for (uint64_t c = 0; c < nchunks; c++) chunk_free(&cvs[c]);
    free(cvs);
    if (per) for (int t = 0; t < T; t++) free(per[t].t);
    free(per);
    free(arr); free(tmp);
    free(g_parent); free(g_sizes); free(g_filtered);
    g_parent = NULL; g_sizes = NULL; g_filtered = NULL;
    free_files(nfiles, f);
    free(f);
    free(scanR); free(thrR); free(hist); free(hd);
    return rc;
}
