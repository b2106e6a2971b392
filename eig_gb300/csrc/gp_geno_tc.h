/* Exact genotype x FP64-panel products on the tensor cores (gp_geno_tc.cu). */
#ifndef GP_GENO_TC_H
#define GP_GENO_TC_H
#include <vector>

#include "gp_internal.h"

/* one FP64 panel P [k][ldp] (device); count = 1: the genotype operand is the allele count
 * {0,1,2}, else the observed mask {0,1}; sign multiplies the panel */
struct gp_tc_panel {
  const double *P;
  int64_t ldp;
  double sign;
  int count;
};

/*
 * sum_over_snps = 1: Y[q][c] = sum_p sum_{s < nk} A_p(samp[q], snprec[s]) sign_p P_p[s][c]
 * sum_over_snps = 0: Y[s][c] = sum_p sum_{q < nsamp} A_p(samp[q], snprec[s]) sign_p P_p[q][c]
 * npanels (1 or 2) panels share the k extent and are concatenated along k with one joint
 * column scale.  Y is device FP64 with row stride ldy; ncols <= 1024.  Uses scratch2.
 */
int gp_geno_panel_tc(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                     const int32_t *d_snprec, int32_t nk, int npanels, const gp_tc_panel *pp,
                     int32_t ncols, double *d_Y, int64_t ldy);
#endif
