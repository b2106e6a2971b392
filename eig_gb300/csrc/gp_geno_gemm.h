/* Products of the decoded genotype matrix with dense panels (FP64 and split-BF16). */
#ifndef GP_GENO_GEMM_H
#define GP_GENO_GEMM_H
#include "gp_internal.h"

/*
 * sum_over_snps = 1:  C[q*ldc + c] = sum_{s<nsnp} T_s[g(samp[q], snprec[s])] * B[s*ldb + c]
 * sum_over_snps = 0:  C[s*ldc + c] = sum_{q<nsamp} T_s[g(samp[q], snprec[s])] * B[q*ldb + c]
 * T_s = d_tab[4*s .. 4*s+3] indexed by the 2-bit code (3 = missing).  All pointers device.
 * Uses scratch2 for split-k partials.
 */
int gp_geno_gemm_f64(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                     const int32_t *d_snprec, const double *d_tab, int32_t nsnp,
                     const double *d_B, int64_t ldb, int32_t ncc, double *d_C, int64_t ldc);

/*
 * The sum over SNPs with usepopsformissing: a missing genotype of sample q takes
 * d_fill[s*npop + d_spop[q]] instead of T_s[3] (T_s[3] when d_spop[q] < 0).
 */
int gp_geno_gemm_f64_fill(gp_ctx *ctx, const int32_t *d_samp, const int32_t *d_spop,
                          int32_t nsamp, const int32_t *d_snprec, const double *d_tab,
                          const double *d_fill, int32_t npop, int32_t nsnp, const double *d_B,
                          int64_t ldb, int32_t ncc, double *d_C, int64_t ldc);

#endif
