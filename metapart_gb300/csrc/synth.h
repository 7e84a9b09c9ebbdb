/* Seeded synthetic metagenome FASTQ generator (see synth.c). */
#ifndef MP_SYNTH_H
#define MP_SYNTH_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { MP_AB_UNIFORM = 0, MP_AB_LOGNORMAL = 1, MP_AB_ZIPF = 2 };

typedef struct {
    uint64_t seed;
    uint64_t n_reads;      /* FASTQ records; even when interleaved */
    int len_choices[4];    /* read length drawn uniformly from these */
    int n_len_choices;
    int n_genomes;
    double glen_lo, glen_hi; /* genome length, log-uniform in [lo, hi] */
    double gc_lo, gc_hi;     /* per-genome GC fraction, uniform in [lo, hi] (0 -> 0.5) */
    int abundance;           /* MP_AB_* */
    double ab_param;         /* log-normal sigma or Zipf exponent */
    double repeat_frac;      /* fraction of each genome overwritten by shared repeats */
    int repeat_len;
    int repeat_pool;
    double sub_rate, n_rate;
    char qual_char;          /* fixed quality char when qual_lo == 0 */
    char qual_lo, qual_hi;   /* uniform quality chars in [lo, hi] */
    int interleaved;         /* 1: mate pairs as consecutive records p<i>/1, p<i>/2 */
    int insert_len;
} mp_synth_spec;

int mp_synth_fastq(const mp_synth_spec *sp, char **out, size_t *out_len);
int mp_synth_fastq_file(const mp_synth_spec *sp, const char *path, size_t *out_len);
void mp_synth_free(char *p);

#ifdef __cplusplus
}
#endif
#endif
