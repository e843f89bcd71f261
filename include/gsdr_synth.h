/* gsdr_synth.h -- seeded synthetic FASTA workloads for tests and benchmarks.
 *
 * Not part of the clustering interface and with no counterpart in the
 * reference (whose own input file is not distributed).  A workload is a set of
 * random seed sequences, each followed by 0..copies_max mutated copies at an
 * identity drawn uniformly from [id_lo, 1], shuffled, written as
 * ">s<index>\n<sequence>\n" records.  Output bytes are identical on every
 * platform for the same configuration.
 */
#ifndef GSDR_SYNTH_H
#define GSDR_SYNTH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { GSDR_LEN_UNIFORM = 0, GSDR_LEN_LOGNORMAL = 1, GSDR_LEN_FIXED = 2, GSDR_LEN_LOGUNIFORM = 3 };
enum { GSDR_MODE_GENERAL = 0, GSDR_MODE_SUBST_FIXED = 1 };

typedef struct {
    int64_t n_reads;        /* total records */
    int64_t n_seeds;        /* seed sequences */
    int32_t len_dist;       /* GSDR_LEN_* */
    int32_t copies_max;     /* copies per seed drawn from 0..copies_max */
    double len_lo, len_hi;  /* bounds (clip for lognormal) */
    double len_median, len_sigma;
    double id_lo;           /* copy identity drawn from [id_lo, 1] */
    double sub_frac;        /* share of edit events that are substitutions */
    int32_t indel_lo, indel_hi;
    double gc_lo, gc_hi;    /* per-seed GC fraction drawn from [gc_lo, gc_hi] */
    int32_t mode;           /* GSDR_MODE_SUBST_FIXED: substitutions only, fixed length */
    int32_t pad_;
    double extra_indel_frac; /* SUBST_FIXED: share of copies with one extra indel */
    uint64_t seed;
} gsdr_synth_cfg;

/* Fill `cfg` with workload recipe 0..4: 0 = 10k reads 200-1000 bp (t 0.95),
 * 1 = 200k reads lognormal lengths, 2 = 2M reads of 150 bp, 3 = 300k reads
 * log-uniform 2-30 kbp, 4 = one serving job (caller sets n_reads / n_seeds). */
void gsdr_synth_preset(int config, gsdr_synth_cfg* cfg);

/* Generate into a malloc'd buffer (free with gsdr_synth_free).  Returns the
 * number of records, or a negative value on bad parameters / no memory. */
int64_t gsdr_synth_generate(const gsdr_synth_cfg* cfg, char** out, int64_t* out_len);
int64_t gsdr_synth_write(const gsdr_synth_cfg* cfg, const char* path);
void gsdr_synth_free(char* p);

#ifdef __cplusplus
}
#endif
#endif
