/*
 * usepopsformissing: a missing genotype takes the mean genotype of the sample's population.
 *
 * In the Gram pass (getcolxz src/eigensrc/smartpca.c:3129-3216 with fvadjust :2236-2279) the
 * population means come from the current rows of each column; the column's mean and fancy
 * scale then run over the observed and the filled values in row order, and the kill rule
 * (:1131-1144) counts the genotypes still missing after the fill.  The SNP weights keep the
 * observed-only table (getcolxf :3564-3592); the sample scores and lsqproj use the filled
 * column's xmean and xfancy (fixxrow src/qpsubs.c:338-348).  lsqproj (:4606-4757) fills from
 * its own population sums over the projected samples that pass the coverage check, with the
 * population index the caller passes per sample.
 *
 * Per pass: the per-population sums and counts of each column are two sums over the rows of
 * the FP64 genotype product (a 0/1/2 table and a 1/1/1 table against the rows' one-hot
 * population matrix; small integers, so exact in any order); then k_popfill, one thread per
 * column, restates the fill and the ordered FP64 sum of fvadjust with the same IEEE
 * operations in the same order, so the table, xmean and xfancy are bit-identical to the
 * reference's.
 */
#include <cuda_runtime.h>

#include "gp_internal.h"
#include "gp_geno_gemm.h"

static int blocks_for(const gp_ctx *ctx, int64_t n, int threads)
{
  int64_t b = (n + threads - 1) / threads;
  if (b > (int64_t)ctx->num_sms * 16) b = (int64_t)ctx->num_sms * 16;
  return b < 1 ? 1 : (int)b;
}

extern "C" int gp_set_row_pops(gp_ctx *ctx, const int32_t *row_pop, int32_t npop)
{
  if (!ctx) return GP_ERR_ARG;
  if (!row_pop || npop <= 0) {
    ctx->npop = 0;
    return GP_OK;
  }
  if (ctx->nrows < 1)
    return gp_fail(ctx, GP_ERR_STATE, "gp_set_row_pops: call gp_set_samples first");
  for (int32_t i = 0; i < ctx->nrows; ++i)
    if (row_pop[i] >= npop)
      return gp_fail(ctx, GP_ERR_ARG, "gp_set_row_pops: row %d population %d >= npop %d", i,
                     row_pop[i], npop);
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  int rc = gp_realloc(ctx, (void **)&ctx->d_rowpop, sizeof(int32_t) * (size_t)ctx->nrows);
  if (rc) return rc;
  GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_rowpop, row_pop, sizeof(int32_t) * (size_t)ctx->nrows,
                         cudaMemcpyHostToDevice, ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->npop = npop;
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  return GP_OK;
}

/* the 4-entry tables of the population sums: genotype value (missing 0) and, when tnum is
 * given, the observed flag */
__global__ void k_pop_tables(double *tsum, double *tnum, int32_t n)
{
  for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    tsum[4 * c] = 0.0;
    tsum[4 * c + 1] = 1.0;
    tsum[4 * c + 2] = 2.0;
    tsum[4 * c + 3] = 0.0;
    if (tnum) {
      tnum[4 * c] = tnum[4 * c + 1] = tnum[4 * c + 2] = 1.0;
      tnum[4 * c + 3] = 0.0;
    }
  }
}

/* B[i*npop + k] = 1 when sample i is in population k and use[i] (NULL: all), else 0 */
__global__ void k_pop_onehot(double *B, const int32_t *pop, const double *use, double min_use,
                             int32_t n, int32_t npop)
{
  const int64_t total = (int64_t)n * npop;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = (int32_t)(idx / npop), k = (int32_t)(idx - (int64_t)i * npop);
    const bool on = pop[i] == k && (!use || use[i] > min_use);
    B[idx] = on ? 1.0 : 0.0;
  }
}

/*
 * One thread per column: the fill and fvadjust's ordered sum over the rows, then the table
 * of the filled column, its population fill values, xmean, xfancy, the count still missing
 * and the kill flag.  k_snp_stats ran before with the missing-count rule off, so cnt holds
 * the observed counts; vtab (the observed-only table of the SNP weights) is cleared for a
 * column the rule kills here.
 */
__global__ void k_popfill(const uint8_t *__restrict__ geno, int64_t rlen,
                          const int32_t *__restrict__ rows, const int32_t *__restrict__ rowpop,
                          int32_t nrows, const int32_t *__restrict__ cols, int32_t ncols,
                          int32_t npop, const double *__restrict__ psum,
                          const double *__restrict__ pnum, gp_xtx_opts o, int32_t *cnt,
                          uint8_t *killed, double *vtab, double *gtab, double *gfill,
                          double *xmean, double *xfancy)
{
  for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncols;
       c += gridDim.x * blockDim.x) {
    const uint8_t *rec = geno + (int64_t)cols[c] * rlen;
    const double *ps = psum + (int64_t)c * npop, *pn = pnum + (int64_t)c * npop;
    double *gt = gtab + 4 * (int64_t)c, *gf = gfill + (int64_t)c * npop;
    for (int32_t k = 0; k < npop; ++k) gf[k] = 0.0;
    gt[0] = gt[1] = gt[2] = gt[3] = 0.0;
    const int32_t c0 = cnt[3 * c], c1 = cnt[3 * c + 1];
    if (c0 < 0) {
      killed[c] = 1; /* no observed genotype: k_snp_stats wrote the reference's outputs */
      continue;
    }
    double ysum = 0.0, ynum = 0.0;
    int32_t miss = 0;
    for (int32_t i = 0; i < nrows; ++i) {
      const int32_t s = rows[i];
      const uint32_t code = (rec[s >> 2] >> ((3 - (s & 3)) * 2)) & 3u;
      if (code != 3u) {
        ysum = __dadd_rn(ysum, (double)code);
        ynum = __dadd_rn(ynum, 1.0);
        continue;
      }
      const int32_t k = rowpop[i];
      if (k >= 0 && pn[k] > 0.5) {
        ysum = __dadd_rn(ysum, __ddiv_rn(ps[k], pn[k]));
        ynum = __dadd_rn(ynum, 1.0);
      } else {
        ++miss;
      }
    }
    const double ymean = __ddiv_rn(ysum, ynum);
    double yfancy = 1.0;
    if (o.fancynorm) {
      double p = __dmul_rn(0.5, ymean);
      if (o.altnormstyle == 0)
        p = __ddiv_rn(__dadd_rn(ysum, 1.0), __dadd_rn(__dmul_rn(2.0, ynum), 2.0));
      const double y = __dmul_rn(p, __dsub_rn(1.0, p));
      if (y > 0.0) yfancy = __ddiv_rn(1.0, __dsqrt_rn(y));
    }
    xmean[c] = __dmul_rn(ymean, yfancy);
    xfancy[c] = yfancy;
    cnt[3 * c + 2] = miss;
    const int32_t t = c0 < c1 ? c0 : c1;
    const int kill = (t < o.minallelecnt) || (miss > o.maxmissing) || (t == 0);
    killed[c] = (uint8_t)kill;
    if (kill) {
      vtab[4 * (int64_t)c] = vtab[4 * (int64_t)c + 1] = vtab[4 * (int64_t)c + 2] = 0.0;
      continue;
    }
    gt[0] = __dmul_rn(-ymean, yfancy);
    gt[1] = __dmul_rn(__dsub_rn(1.0, ymean), yfancy);
    gt[2] = __dmul_rn(__dsub_rn(2.0, ymean), yfancy);
    for (int32_t k = 0; k < npop; ++k)
      if (pn[k] > 0.5) gf[k] = __dmul_rn(__dsub_rn(__ddiv_rn(ps[k], pn[k]), ymean), yfancy);
  }
}

int gp_popfill_pass(gp_ctx *ctx, const gp_xtx_opts *o)
{
  const int32_t n = ctx->nrows, nc = ctx->ncols, P = ctx->npop;
  int rc = gp_realloc(ctx, (void **)&ctx->d_gtab, sizeof(double) * 4 * (size_t)nc);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_gfill, sizeof(double) * (size_t)nc * P);
  if (rc) return rc;
  const size_t ntab = 4 * (size_t)nc, nB = (size_t)n * P, nps = (size_t)nc * P;
  double *base;
  rc = gp_scratch(ctx, sizeof(double) * (2 * ntab + nB + 2 * nps), (void **)&base);
  if (rc) return rc;
  double *tsum = base, *tnum = tsum + ntab, *B = tnum + ntab, *psum = B + nB, *pnum = psum + nps;
  k_pop_tables<<<blocks_for(ctx, nc, 256), 256, 0, ctx->stream>>>(tsum, tnum, nc);
  GP_LAUNCH_CHECK(ctx, "k_pop_tables");
  k_pop_onehot<<<blocks_for(ctx, (int64_t)n * P, 256), 256, 0, ctx->stream>>>(
      B, ctx->d_rowpop, NULL, 0.0, n, P);
  GP_LAUNCH_CHECK(ctx, "k_pop_onehot");
  rc = gp_geno_gemm_f64(ctx, 0, ctx->d_rows, n, ctx->d_cols, tsum, nc, B, P, P, psum, P);
  if (!rc) rc = gp_geno_gemm_f64(ctx, 0, ctx->d_rows, n, ctx->d_cols, tnum, nc, B, P, P, pnum, P);
  if (rc) return rc;
  gp_xtx_opts oo = *o;
  k_popfill<<<blocks_for(ctx, nc, 128), 128, 0, ctx->stream>>>(
      ctx->d_geno, ctx->rlen_dev, ctx->d_rows, ctx->d_rowpop, n, ctx->d_cols, nc, P, psum, pnum,
      oo, ctx->d_cnt, ctx->d_killed, ctx->d_vtab, ctx->d_gtab, ctx->d_gfill, ctx->d_xmean,
      ctx->d_xfancy);
  GP_LAUNCH_CHECK(ctx, "k_popfill");
  return GP_OK;
}

/* of[s*npop + k] = 1 and rf[s*npop + k] = fixxrow(xnum/xden) where xden > 0.1, else 0 */
__global__ void k_lsq_fill_tables(const double *xnum, const double *xden, const int32_t *kept,
                                  const double *xmean, const double *xfancy, int32_t nk,
                                  int32_t npop, double *of, double *rf)
{
  const int64_t total = (int64_t)nk * npop;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = (int32_t)(idx / npop), c = kept[s];
    double o1 = 0.0, r1 = 0.0;
    if (xden[idx] > 0.1) {
      const double x = __dmul_rn(__ddiv_rn(xnum[idx], xden[idx]), xfancy[c]);
      o1 = 1.0;
      r1 = (x < -0.001) ? 0.0 : __dsub_rn(x, xmean[c]);
    }
    of[idx] = o1;
    rf[idx] = r1;
  }
}

size_t gp_lsq_fill_work_bytes(int32_t nproj, int32_t nk, int32_t npop)
{
  return sizeof(double) * ((size_t)nproj + 5 * (size_t)nk + (size_t)nproj * npop +
                           4 * (size_t)nk * npop) + 1024;
}

__global__ void k_set_value(double *x, int64_t n, double v)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

/*
 * lsqproj's population fill tables (smartpca.c:4631-4677): raw[q] = observed kept genotypes
 * of sample q; xnum/xden = per-population sums and counts over the samples with a
 * population and raw > K (the coverage check: the others are "ignored (insufficient data"
 * before the sums); of/rf [nk*npop] the observed flag and the fixxrow value of the fill.
 * d_ot = the kept columns' observed-flag tables {1,1,1,0}.  work: gp_lsq_fill_work_bytes.
 */
int gp_lsq_fill_tables(gp_ctx *ctx, const int32_t *d_samp, const int32_t *d_spop, int32_t nproj,
                       int32_t npop, int32_t K, const int32_t *d_snprec, const double *d_ot,
                       int32_t nk, void *work, double **d_raw, double **d_of, double **d_rf)
{
  const size_t nkp = (size_t)nk * npop;
  double *raw = (double *)work, *ones = raw + nproj, *tsum = ones + nk;
  double *B = tsum + 4 * (size_t)nk, *xnum = B + (size_t)nproj * npop, *xden = xnum + nkp;
  double *of = xden + nkp, *rf = of + nkp;
  *d_raw = raw;
  *d_of = of;
  *d_rf = rf;
  k_set_value<<<blocks_for(ctx, nk, 256), 256, 0, ctx->stream>>>(ones, nk, 1.0);
  GP_LAUNCH_CHECK(ctx, "k_set_value");
  k_pop_tables<<<blocks_for(ctx, nk, 256), 256, 0, ctx->stream>>>(tsum, NULL, nk);
  GP_LAUNCH_CHECK(ctx, "k_pop_tables");
  int rc = gp_geno_gemm_f64(ctx, 1, d_samp, nproj, d_snprec, d_ot, nk, ones, 1, 1, raw, 1);
  if (rc) return rc;
  k_pop_onehot<<<blocks_for(ctx, (int64_t)nproj * npop, 256), 256, 0, ctx->stream>>>(
      B, d_spop, raw, (double)K + 0.5, nproj, npop);
  GP_LAUNCH_CHECK(ctx, "k_pop_onehot");
  rc = gp_geno_gemm_f64(ctx, 0, d_samp, nproj, d_snprec, tsum, nk, B, npop, npop, xnum, npop);
  if (!rc) rc = gp_geno_gemm_f64(ctx, 0, d_samp, nproj, d_snprec, d_ot, nk, B, npop, npop, xden,
                                 npop);
  if (rc) return rc;
  k_lsq_fill_tables<<<blocks_for(ctx, (int64_t)nkp, 256), 256, 0, ctx->stream>>>(
      xnum, xden, ctx->d_kept, ctx->d_xmean, ctx->d_xfancy, nk, npop, of, rf);
  GP_LAUNCH_CHECK(ctx, "k_lsq_fill_tables");
  return GP_OK;
}
