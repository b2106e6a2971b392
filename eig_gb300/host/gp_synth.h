/* Seeded Balding–Nichols genotype generator (packedancestrymap records). */
#ifndef GP_SYNTH_H
#define GP_SYNTH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GP_SYNTH_MAXPOPS 64

typedef struct {
  int64_t nsnp;             /* M */
  int32_t nind;             /* N: sum(pop_sizes) unmixed samples, the rest two-way admixed */
  int32_t npops;
  const int32_t *pop_sizes; /* npops entries */
  const double *fst;        /* npops entries, F of each population */
  double p_lo, p_hi;        /* ancestral allele frequency range */
  double miss_lo, miss_hi;  /* per-sample missing rate ~ U(miss_lo, miss_hi); equal = fixed */
  uint64_t seed;
} gp_synth_spec;

int64_t gp_packed_rlen(int32_t nind);
int32_t gp_hash_string(const char *s);
int32_t gp_hash_list(const char *const *ids, int64_t n);

/* Per-sample population assignment, admixture fraction and missing rate. */
int gp_synth_assign(const gp_synth_spec *sp, int32_t *pop_a, int32_t *pop_b, double *mix,
                    double *miss);

/* Fill nsnp records of rlen bytes; pop_of_sample (may be NULL) receives the population of
 * each sample (npops for admixed samples). */
int gp_synth_records(const gp_synth_spec *sp, uint8_t *records, int64_t rlen,
                     int32_t *pop_of_sample, int nthreads);

/* New samples of the spec's populations (the same per-SNP population frequencies as
 * gp_synth_records with sp->seed; assignment, admixture, missingness and genotypes drawn
 * with sample_seed): sp->nind rows of row_bytes bytes, sample n's code at panel SNP k
 * (record snp_index[k]) in byte k>>2, bits (3-(k&3))*2, padded with code 3. */
int gp_synth_sample_rows(const gp_synth_spec *sp, uint64_t sample_seed, const int64_t *snp_index,
                         int64_t nk, int64_t row_bytes, uint8_t *rows, int32_t *pop_of_sample,
                         int nthreads);

/* Write prefix.geno (packed, with header hashes), prefix.snp and prefix.ind. */
int gp_synth_write_dataset(const gp_synth_spec *sp, const char *prefix, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
