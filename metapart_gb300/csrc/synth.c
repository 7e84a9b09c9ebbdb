/*
 * Seeded synthetic metagenome FASTQ generator.
 *
 * Produces the read sets the benchmark workloads are defined on: reads sampled
 * from synthetic genomes (i.i.d. bases with a per-genome GC fraction, optional
 * shared repeat elements), genome abundances uniform / log-normal / Zipf,
 * uniform substitution errors, N at a given rate, and a fixed or uniformly
 * random quality string.  Output is single-end or interleaved paired-end FASTQ
 * with '\n' line endings and quality length == sequence length, the record
 * layout the reference parser assumes (genHistograms.c:60-80,
 * metapart.c:296-369).
 *
 * Every genome and every read draws from its own counter-based random stream
 * (splitmix64 of seed and index), so the bytes do not depend on the number of
 * OpenMP threads.  A quality line never starts with '+' (the reference chunk
 * indexer, genFastqIdx.c:258-302, would take such a line for a separator).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "synth.h"

static inline uint64_t sm64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t mix(uint64_t a, uint64_t b)
{
    uint64_t s = a ^ (b * 0xD1B54A32D192ED03ull);
    return sm64(&s);
}
/* uniform double in [0,1) */
static inline double u01(uint64_t *s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }
static inline uint64_t ubelow(uint64_t *s, uint64_t n) { return n ? (uint64_t)(u01(s) * (double)n) % n : 0; }
static double gauss(uint64_t *s)
{
    double u1 = u01(s), u2 = u01(s);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

static const char BASES[4] = {'A', 'C', 'G', 'T'};
static inline char comp(char c)
{
    switch (c) { case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C'; case 'T': return 'A'; }
    return 'N';
}
static inline char rand_base(uint64_t *s, double gc)
{
    double u = u01(s);
    if (u < gc) return (u < gc * 0.5) ? 'G' : 'C';
    return (u < gc + (1.0 - gc) * 0.5) ? 'A' : 'T';
}

typedef struct {
    char **seq;
    uint64_t *len;
    double *cum; /* cumulative sampling weight */
    int n;
} genome_set;

static void free_genomes(genome_set *g)
{
    if (g->seq) for (int i = 0; i < g->n; i++) free(g->seq[i]);
    free(g->seq); free(g->len); free(g->cum);
}

static int make_genomes(const mp_synth_spec *sp, genome_set *g)
{
    int n = sp->n_genomes > 0 ? sp->n_genomes : 1;
    g->n = n;
    g->seq = (char **)calloc((size_t)n, sizeof(char *));
    g->len = (uint64_t *)calloc((size_t)n, sizeof(uint64_t));
    g->cum = (double *)calloc((size_t)n, sizeof(double));
    if (!g->seq || !g->len || !g->cum) return -1;
    /* shared repeat pool */
    int pool = (sp->repeat_frac > 0 && sp->repeat_len > 0) ? (sp->repeat_pool > 0 ? sp->repeat_pool : 64) : 0;
    char *rep = NULL;
    if (pool) {
        rep = (char *)malloc((size_t)pool * (size_t)sp->repeat_len);
        if (!rep) return -1;
        for (int r = 0; r < pool; r++) {
            uint64_t s = mix(sp->seed ^ 0x5EEDull, 0x100000000ull + (uint64_t)r);
            for (int j = 0; j < sp->repeat_len; j++) rep[(size_t)r * sp->repeat_len + j] = BASES[sm64(&s) & 3];
        }
    }
    double *w = (double *)malloc((size_t)n * sizeof(double));
    int fail = 0;
    if (!w) { free(rep); return -1; }
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) {
        uint64_t s = mix(sp->seed, 0x200000000ull + (uint64_t)i);
        double lo = sp->glen_lo > 0 ? sp->glen_lo : 50000, hi = sp->glen_hi > lo ? sp->glen_hi : lo;
        double L = (hi > lo) ? exp(log(lo) + u01(&s) * (log(hi) - log(lo))) : lo;
        uint64_t len = (uint64_t)L;
        double gc = (sp->gc_hi > sp->gc_lo) ? sp->gc_lo + u01(&s) * (sp->gc_hi - sp->gc_lo)
                                            : (sp->gc_lo > 0 ? sp->gc_lo : 0.5);
        char *q = (char *)malloc(len + 1);
        if (!q) { fail = 1; continue; }
        for (uint64_t j = 0; j < len; j++) q[j] = rand_base(&s, gc);
        if (pool) {
            /* overwrite repeat_frac of the genome with copies of pooled repeats */
            uint64_t ncopies = (uint64_t)(sp->repeat_frac * (double)len / (double)sp->repeat_len);
            for (uint64_t c = 0; c < ncopies && len > (uint64_t)sp->repeat_len; c++) {
                uint64_t pos = ubelow(&s, len - (uint64_t)sp->repeat_len);
                int r = (int)ubelow(&s, (uint64_t)pool);
                memcpy(q + pos, rep + (size_t)r * sp->repeat_len, (size_t)sp->repeat_len);
            }
        }
        q[len] = 0;
        g->seq[i] = q;
        g->len[i] = len;
        double a = 1.0;
        if (sp->abundance == MP_AB_LOGNORMAL) a = exp(sp->ab_param * gauss(&s));
        else if (sp->abundance == MP_AB_ZIPF) a = 1.0 / pow((double)(i + 1), sp->ab_param);
        w[i] = a * (double)len;
    }
    free(rep);
    if (fail) { free(w); return -1; }
    double acc = 0;
    for (int i = 0; i < n; i++) { acc += w[i]; g->cum[i] = acc; }
    for (int i = 0; i < n; i++) g->cum[i] /= acc;
    free(w);
    return 0;
}

static int pick_genome(const genome_set *g, double u)
{
    int lo = 0, hi = g->n - 1;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (g->cum[mid] > u) hi = mid; else lo = mid + 1;
    }
    return lo;
}

static int read_len_of(const mp_synth_spec *sp, uint64_t *s)
{
    if (sp->n_len_choices <= 1) return sp->len_choices[0];
    return sp->len_choices[ubelow(s, (uint64_t)sp->n_len_choices)];
}

/* writes one record; returns bytes written */
static size_t emit_record(char *o, const char *name, size_t nlen, const char *bases, int L,
                          const mp_synth_spec *sp, uint64_t *s)
{
    size_t p = 0;
    o[p++] = '@';
    memcpy(o + p, name, nlen); p += nlen;
    o[p++] = '\n';
    memcpy(o + p, bases, (size_t)L); p += (size_t)L;
    o[p++] = '\n';
    o[p++] = '+';
    o[p++] = '\n';
    if (sp->qual_lo && sp->qual_hi > sp->qual_lo) {
        int span = sp->qual_hi - sp->qual_lo + 1;
        for (int j = 0; j < L; j++) {
            char c;
            do { c = (char)(sp->qual_lo + (int)ubelow(s, (uint64_t)span)); } while (j == 0 && c == '+');
            o[p++] = c;
        }
    } else {
        char c = sp->qual_char ? sp->qual_char : 'I';
        if (c == '+') c = 'I';
        memset(o + p, c, (size_t)L); p += (size_t)L;
    }
    o[p++] = '\n';
    return p;
}

/* sample a fragment of length flen from genome gi; fills buf (forward strand) */
static void sample_fragment(const genome_set *g, int gi, int flen, uint64_t *s, char *buf)
{
    uint64_t glen = g->len[gi];
    if ((uint64_t)flen >= glen) {
        for (int j = 0; j < flen; j++) buf[j] = g->seq[gi][(uint64_t)j % glen];
        return;
    }
    uint64_t pos = ubelow(s, glen - (uint64_t)flen + 1);
    memcpy(buf, g->seq[gi] + pos, (size_t)flen);
}

static void mutate(char *b, int L, const mp_synth_spec *sp, uint64_t *s)
{
    for (int j = 0; j < L; j++) {
        if (sp->sub_rate > 0 && u01(s) < sp->sub_rate) {
            char c;
            do { c = BASES[sm64(s) & 3]; } while (c == b[j]);
            b[j] = c;
        }
        if (sp->n_rate > 0 && u01(s) < sp->n_rate) b[j] = 'N';
    }
}

static size_t record_bound(const mp_synth_spec *sp, int L)
{
    return (size_t)L * 2 + 64;
}

int mp_synth_fastq(const mp_synth_spec *sp, char **out, size_t *out_len)
{
    if (!sp || !out || !out_len || sp->n_reads == 0 || sp->len_choices[0] <= 0) return -1;
    if (sp->interleaved && (sp->n_reads & 1)) return -1;
    genome_set g = {0};
    if (make_genomes(sp, &g) != 0) { free_genomes(&g); return -2; }
    int maxL = 0;
    for (int i = 0; i < (sp->n_len_choices > 0 ? sp->n_len_choices : 1); i++)
        if (sp->len_choices[i] > maxL) maxL = sp->len_choices[i];
    uint64_t nunits = sp->interleaved ? sp->n_reads / 2 : sp->n_reads;
    int per_unit = sp->interleaved ? 2 : 1;
    /* per-unit byte counts first (pass 1 computes lengths deterministically), then offsets */
    size_t *ulen = (size_t *)malloc((size_t)nunits * sizeof(size_t));
    if (!ulen) { free_genomes(&g); return -2; }
#pragma omp parallel for schedule(static)
    for (uint64_t u = 0; u < nunits; u++) {
        uint64_t s = mix(sp->seed, 0x300000000ull + u);
        int L = read_len_of(sp, &s);
        char name[48];
        int nl = sp->interleaved ? snprintf(name, sizeof name, "p%llu/1", (unsigned long long)u)
                                 : snprintf(name, sizeof name, "r%llu", (unsigned long long)u);
        ulen[u] = (size_t)per_unit * ((size_t)nl + 6 + 2 * (size_t)L);
    }
    size_t total = 0;
    for (uint64_t u = 0; u < nunits; u++) { size_t t = ulen[u]; ulen[u] = total; total += t; }
    char *o = (char *)malloc(total + 16);
    if (!o) { free(ulen); free_genomes(&g); return -2; }
    int insert = sp->insert_len > 0 ? sp->insert_len : 2 * maxL + 100;
#pragma omp parallel
    {
        char *frag = (char *)malloc((size_t)(insert > maxL ? insert : maxL) + 8);
        char *b1 = (char *)malloc((size_t)maxL + 8), *b2 = (char *)malloc((size_t)maxL + 8);
#pragma omp for schedule(static)
        for (uint64_t u = 0; u < nunits; u++) {
            uint64_t s = mix(sp->seed, 0x300000000ull + u);
            int L = read_len_of(sp, &s);
            int gi = pick_genome(&g, u01(&s));
            char name[48];
            size_t p = ulen[u];
            if (!sp->interleaved) {
                sample_fragment(&g, gi, L, &s, frag);
                if (sm64(&s) & 1) for (int j = 0; j < L; j++) b1[j] = comp(frag[L - 1 - j]);
                else memcpy(b1, frag, (size_t)L);
                mutate(b1, L, sp, &s);
                int nl = snprintf(name, sizeof name, "r%llu", (unsigned long long)u);
                p += emit_record(o + p, name, (size_t)nl, b1, L, sp, &s);
            } else {
                int fl = insert < L ? L : insert;
                sample_fragment(&g, gi, fl, &s, frag);
                int flip = (int)(sm64(&s) & 1);
                if (flip) { for (int j = 0; j < fl / 2; j++) { char t = comp(frag[j]); frag[j] = comp(frag[fl - 1 - j]); frag[fl - 1 - j] = t; }
                            if (fl & 1) frag[fl / 2] = comp(frag[fl / 2]); }
                memcpy(b1, frag, (size_t)L);
                for (int j = 0; j < L; j++) b2[j] = comp(frag[fl - 1 - j]);
                mutate(b1, L, sp, &s);
                mutate(b2, L, sp, &s);
                int nl = snprintf(name, sizeof name, "p%llu/1", (unsigned long long)u);
                p += emit_record(o + p, name, (size_t)nl, b1, L, sp, &s);
                nl = snprintf(name, sizeof name, "p%llu/2", (unsigned long long)u);
                p += emit_record(o + p, name, (size_t)nl, b2, L, sp, &s);
            }
        }
        free(frag); free(b1); free(b2);
    }
    free(ulen);
    free_genomes(&g);
    (void)record_bound;
    *out = o;
    *out_len = total;
    return 0;
}

void mp_synth_free(char *p) { free(p); }

int mp_synth_fastq_file(const mp_synth_spec *sp, const char *path, size_t *out_len)
{
    char *buf = NULL;
    size_t n = 0;
    int rc = mp_synth_fastq(sp, &buf, &n);
    if (rc) return rc;
    FILE *f = fopen(path, "wb");
    if (!f) { free(buf); return -3; }
    size_t w = fwrite(buf, 1, n, f);
    fclose(f);
    free(buf);
    if (w != n) return -3;
    if (out_len) *out_len = n;
    return 0;
}
