/* Exact genotype x FP64-panel products on the tensor cores (gp_geno_tc.cu). */
#ifndef GP_GENO_TC_H
#define GP_GENO_TC_H
#include <cuda.h>
#include <cuda_fp16.h>
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

/* A genotype code operand: rows of ldc bytes of 2-bit codes (MSB first, 3 -> 0); output
 * row r reads code row row_map[r] (or r); k0 = the k extent of one panel. */
struct gp_tc_codes {
  const uint8_t *codes;
  int64_t ldc;
  const int32_t *row_map;
  int32_t nrows;
  int32_t k0;
};

/* bytes of the code operand built by gp_tc_build_codes: rows_pad * ldc */
int gp_tc_code_bytes(int sum_over_snps, int32_t nsamp, int32_t nk, int64_t *ldc, int32_t *rows_pad);
int gp_tc_build_codes(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                      const int32_t *d_snprec, int32_t nk, uint8_t *codes, gp_tc_codes *out);
/* a panel cut into fp16 slices once (B operand + column exponents + its tensor map) */
struct gp_tc_prepared {
  __half *B;
  int32_t *expo;
  int32_t ncols, ncols4, ncols4_pad, npanels, kb0, k0;
  int64_t ldb;
  uint64_t lut_lo, lut_hi;
  CUtensorMap tmb;
};
size_t gp_tc_prepared_bytes(int npanels, int32_t ncols, int32_t k0);
/* slice the panels into caller storage of gp_tc_prepared_bytes bytes (device) */
int gp_tc_prepare(gp_ctx *ctx, int npanels, const gp_tc_panel *pp, int32_t ncols, int32_t k0,
                  void *storage, gp_tc_prepared *out);
/* Y[r][c] = products of the code operand with a prepared panel; sync = 0 leaves the work
 * queued on ctx->stream and neither clears nor reads ctx->d_err (the caller does both) */
int gp_tc_apply(gp_ctx *ctx, const gp_tc_codes *A, const gp_tc_prepared *P, double *d_Y,
                int64_t ldy, int sync);

/* The batch a device-resident loop works on: nrows code rows at codes (ring position row0
 * of the pool), requests [req_begin, req_end) of the loop's queue.  Written on the device
 * by the loop's batch former and read by the kernels at run time, so that one captured
 * launch serves every batch. */
struct gp_tc_batch {
  const uint8_t *codes;
  int32_t nrows;
  int32_t pad;
  int64_t row0, req_begin, req_end;
};
/* gp_tc_apply inside a loop body: the rows come from db at run time (at most max_rows, row
 * stride ldc); Z holds max_rows * P->ncols4_pad doubles of the caller's; errors of the
 * bounded waits go to ctx->d_err */
int gp_tc_apply_dev(gp_ctx *ctx, const gp_tc_batch *db, int32_t max_rows, int64_t ldc,
                    const gp_tc_prepared *P, double *Z, double *d_Y, int64_t ldy);

/* the code operand of gp_geno_panel_tc (built into scratch4, or the resident records when a
 * SNP-major operand covers every sample in order) */
int gp_tc_codes_for(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                    const int32_t *d_snprec, int32_t nk, gp_tc_codes *out);
/* Y[r][c] = sum_p sum_k A(r, k) sign_p P_p[k][c] with a prepared code operand */
int gp_geno_panel_tc_codes(gp_ctx *ctx, const gp_tc_codes *A, int npanels, const gp_tc_panel *pp,
                           int32_t ncols, double *d_Y, int64_t ldy);

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
