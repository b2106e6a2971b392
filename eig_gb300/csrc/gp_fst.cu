/*
 * Fst between populations after the PCA (dofstxx src/eigensrc/smartpca.c:2830-2878 ->
 * dofstnumx src/qpsubs.c:2488-2720, fstcolyy :1205-1345, wjackest :2793-2858).
 *
 * Device: per population allele counts of every column of the last pass over the current rows
 * (c0 = sum g, c1 = sum (2 - g) over the observed genotypes of the population's rows), from
 * the packed records with one 2-bit selection mask per population, the same popcount
 * arithmetic as the per-SNP counts of gp_xtx (k_snp_stats).  Host: the reference's estimator
 * per column and population pair, the per-block sums in column order, the delete-one-block
 * estimates and the weighted block jackknife, with the reference's operation order.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include <vector>

#include "gp_internal.h"

/* masks[p][w]: 0b11 under every row of population p (xtypes[r] == p) */
__global__ void k_pop_masks(uint32_t *masks, int64_t nwords, const int32_t *rows,
                            const int32_t *xtypes, int32_t nrows, int32_t numeg)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = xtypes[i];
    if (p < 0 || p >= numeg) continue;
    const int32_t k = rows[i];
    const uint32_t shift = (uint32_t)((k & 15) >> 2) * 8u + (3u - (uint32_t)(k & 3)) * 2u;
    atomicOr(&masks[(int64_t)p * nwords + (k >> 4)], 3u << shift);
  }
}

/* counts[(c * numeg + p) * 2 + {0, 1}]: one warp per column, populations in turn */
__global__ void k_pop_counts(const uint8_t *__restrict__ geno, int64_t rlen_dev,
                             const uint32_t *__restrict__ masks, const int32_t *__restrict__ cols,
                             int32_t ncols, int32_t numeg, int32_t *counts)
{
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t words = rlen_dev >> 2;
  for (int64_t c = warp; c < ncols; c += nw) {
    const uint32_t *rec = (const uint32_t *)(geno + (int64_t)cols[c] * rlen_dev);
    for (int32_t p = 0; p < numeg; ++p) {
      const uint32_t *m = masks + (int64_t)p * words;
      int32_t sumg = 0, nobs = 0;
      for (int64_t i = lane; i < words; i += 32) {
        const uint32_t sel = __ldg(m + i) & 0x55555555u;
        if (!sel) continue;
        const uint32_t w = __ldg(rec + i);
        const uint32_t hi = (w >> 1) & 0x55555555u, lo = w & 0x55555555u;
        const uint32_t obs = sel & ~(hi & lo);
        sumg += 2 * __popc(hi & obs) + __popc(lo & obs);
        nobs += __popc(obs);
      }
      for (int off = 16; off; off >>= 1) {
        sumg += __shfl_down_sync(0xffffffffu, sumg, off);
        nobs += __shfl_down_sync(0xffffffffu, nobs, off);
      }
      if (lane == 0) {
        counts[(c * numeg + p) * 2] = sumg;
        counts[(c * numeg + p) * 2 + 1] = 2 * nobs - sumg;
      }
    }
  }
}

/* wjackestx (src/qpsubs.c:2818-2858): weighted block jackknife, blocks of weight >= 1e-6 */
static void wjack(double *est, double *sig, double mean, const std::vector<double> &jmean_all,
                  const std::vector<double> &jwt_all)
{
  std::vector<double> jmean, jwt;
  for (size_t i = 0; i < jwt_all.size(); ++i) {
    if (jwt_all[i] < 1.0e-6) continue;
    jmean.push_back(jmean_all[i]);
    jwt.push_back(jwt_all[i]);
  }
  const int g = (int)jwt.size();
  if (g <= 1) {
    *est = mean;
    *sig = 0.0;
    return;
  }
  double yn = 0.0;
  for (int k = 0; k < g; ++k) yn += jwt[k];
  double sdiff = 0.0, dot = 0.0;
  for (int k = 0; k < g; ++k) sdiff += -(jmean[k] + -mean);
  for (int k = 0; k < g; ++k) dot += jwt[k] * jmean[k];
  const double jackest = sdiff + dot / yn;
  double var = 0.0;
  for (int k = 0; k < g; ++k) {
    const double hh = yn / jwt[k];
    const double w1 = hh + -1.0;
    double xt = hh * mean - w1 * jmean[k];
    xt = xt + -jackest;
    xt = xt * xt;
    var += xt / w1;
  }
  *est = jackest;
  *sig = sqrt(var / (double)g);
}

extern "C" int gp_fst(gp_ctx *ctx, const int32_t *xtypes, int32_t numeg, const int32_t *snp_block,
                      int32_t nblocks, double *fstmean, double *fstans, double *fstsd,
                      int32_t *fstnum)
{
  if (!ctx || !xtypes || numeg < 1 || !snp_block || nblocks < 1)
    return GP_ERR_ARG;
  /* the kill flags of the current rows and columns come from their gp_xtx; gp_eigvecs
   * consumes the Gram but keeps them */
  if (!ctx->xtx_valid && !ctx->eig_valid)
    return gp_fail(ctx, GP_ERR_STATE, "gp_fst: no pass to take the columns from (gp_xtx first)");
  const int32_t n = ctx->nrows, nc = ctx->ncols, E = numeg;
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t words = ctx->rlen_dev / 4;
  const size_t mask_bytes = sizeof(uint32_t) * (size_t)words * (size_t)E;
  const size_t xt_bytes = (sizeof(int32_t) * (size_t)n + 255) & ~(size_t)255;
  /* columns in chunks so that the counts of a chunk stay within 64 MB whatever numeg is
   * (GP_FST_CHUNK_COLS sets a smaller chunk) */
  int64_t chunk = ((int64_t)64 << 20) / ((int64_t)8 * E);
  const char *cenv = getenv("GP_FST_CHUNK_COLS");
  if (cenv && atoll(cenv) > 0 && atoll(cenv) < chunk) chunk = atoll(cenv);
  if (chunk < 1) chunk = 1;
  if (chunk > nc) chunk = nc > 0 ? nc : 1;
  const size_t cnt_bytes = sizeof(int32_t) * 2 * (size_t)E * (size_t)chunk;
  uint8_t *base;
  int rc = gp_scratch(ctx, ((mask_bytes + 255) & ~(size_t)255) + xt_bytes + cnt_bytes + 256,
                      (void **)&base);
  if (rc) return rc;
  uint32_t *d_masks = (uint32_t *)base;
  int32_t *d_xt = (int32_t *)(base + ((mask_bytes + 255) & ~(size_t)255));
  int32_t *d_cnt = (int32_t *)((uint8_t *)d_xt + xt_bytes);
  GP_CUDA(ctx, cudaMemsetAsync(d_masks, 0, mask_bytes, ctx->stream));
  GP_CUDA(ctx, gp_memcpy(ctx, d_xt, xtypes, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice,
                         ctx->stream));
  {
    int blocks = (n + 255) / 256;
    if (blocks > ctx->num_sms * 8) blocks = ctx->num_sms * 8;
    k_pop_masks<<<blocks < 1 ? 1 : blocks, 256, 0, ctx->stream>>>(d_masks, words, ctx->d_rows, d_xt,
                                                                  n, E);
    GP_LAUNCH_CHECK(ctx, "k_pop_masks");
  }
  std::vector<int32_t> cnt((size_t)2 * E * (size_t)chunk), cols((size_t)nc);
  std::vector<uint8_t> killed((size_t)nc);
  GP_CUDA(ctx, gp_memcpy(ctx, cols.data(), ctx->d_cols, sizeof(int32_t) * (size_t)nc,
                         cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, gp_memcpy(ctx, killed.data(), ctx->d_killed, (size_t)nc, cudaMemcpyDeviceToHost,
                         ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));

  /* per-block sums in column order (dofstnumx :2554-2620, fstmode YES: top += n, bot += d) */
  const size_t EE = (size_t)E * E;
  std::vector<double> btop((size_t)nblocks * EE, 0.0), bbot((size_t)nblocks * EE, 0.0);
  std::vector<double> wj((size_t)nblocks, 0.0);
  std::vector<int32_t> num(EE, 0);
  for (int32_t c0 = 0; c0 < nc; c0 += (int32_t)chunk) {
    const int32_t ncc = nc - c0 < chunk ? nc - c0 : (int32_t)chunk;
    int64_t blocks = ((int64_t)ncc * 32 + 255) / 256;
    if (blocks > (int64_t)ctx->num_sms * 16) blocks = (int64_t)ctx->num_sms * 16;
    if (blocks < 1) blocks = 1;
    k_pop_counts<<<(unsigned)blocks, 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, d_masks,
                                                            ctx->d_cols + c0, ncc, E, d_cnt);
    GP_LAUNCH_CHECK(ctx, "k_pop_counts");
    GP_CUDA(ctx, gp_memcpy(ctx, cnt.data(), d_cnt, sizeof(int32_t) * 2 * (size_t)E * ncc,
                           cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int32_t c = c0; c < c0 + ncc; ++c) {
      if (killed[(size_t)c]) continue;
      const int32_t bnum = snp_block[cols[(size_t)c]];
      if (bnum < 0) continue;
      if (bnum >= nblocks) return gp_fail(ctx, GP_ERR_ARG, "gp_fst: block %d >= %d", bnum, nblocks);
      wj[(size_t)bnum] += 1.0;
      double *top = &btop[(size_t)bnum * EE], *bot = &bbot[(size_t)bnum * EE];
      const int32_t *cc = &cnt[(size_t)(c - c0) * E * 2];
      for (int32_t a = 0; a < E; ++a) {
        for (int32_t b = a + 1; b < E; ++b) {
          /* fstcolyy (:1301-1337) */
          const double ya = cc[2 * a], yb = cc[2 * a + 1], yaa = cc[2 * b], ybb = cc[2 * b + 1];
          const double zz = yaa + ybb, z = ya + yb;
          if ((z < 1.5) || (zz < 1.5)) continue;
          double yt = ya + yb;
          const double p1 = ya / yt;
          const double h1 = ya * yb / (yt * (yt - 1.0));
          yt = yaa + ybb;
          const double p2 = yaa / yt;
          const double h2 = yaa * ybb / (yt * (yt - 1.0));
          double en = (p1 - p2) * (p1 - p2);
          en -= h1 / z;
          en -= h2 / zz;
          double ed = en;
          ed += h1;
          ed += h2;
          if (ed < 0.0) continue;
          const size_t k = (size_t)a * E + b;
          ++num[k];
          top[k] += en;
          bot[k] += ed;
        }
      }
    }
  }
  /* totals, delete-one-block estimates, jackknife (:2642-2686) */
  std::vector<double> gtop(EE, 0.0), gbot(EE, 0.0);
  for (int32_t k = 0; k < nblocks; ++k)
    for (size_t i = 0; i < EE; ++i) {
      gtop[i] += btop[(size_t)k * EE + i];
      gbot[i] += bbot[(size_t)k * EE + i];
    }
  std::vector<double> djk((size_t)nblocks * EE);
  for (int32_t k = 0; k < nblocks; ++k)
    for (size_t i = 0; i < EE; ++i) {
      const double wt = gtop[i] - btop[(size_t)k * EE + i];
      const double wb = (gbot[i] - bbot[(size_t)k * EE + i]) + 1.0e-10;
      djk[(size_t)k * EE + i] = wt / wb;
    }
  std::vector<double> fst(EE);
  for (size_t i = 0; i < EE; ++i) fst[i] = gtop[i] / (gbot[i] + 1.0e-10);
  for (size_t i = 0; i < EE; ++i) {
    if (fstans) fstans[i] = 0.0;
    if (fstsd) fstsd[i] = 0.0;
    if (fstmean) fstmean[i] = fst[i];
    if (fstnum) fstnum[i] = 0;
  }
  std::vector<double> dj((size_t)nblocks);
  for (int32_t i = 0; i < E; ++i) {
    for (int32_t j = i + 1; j < E; ++j) {
      const size_t k = (size_t)i * E + j;
      for (int32_t b = 0; b < nblocks; ++b) dj[(size_t)b] = djk[(size_t)b * EE + k];
      double jest = fst[k], jsig = 0.0;
      if (nblocks > 1) wjack(&jest, &jsig, fst[k], dj, wj);
      if (fstans) fstans[k] = fstans[(size_t)j * E + i] = jest;
      if (fstsd) fstsd[k] = fstsd[(size_t)j * E + i] = jsig;
      if (fstnum) fstnum[k] = fstnum[(size_t)j * E + i] = num[k];
    }
  }
  return GP_OK;
}

/* setblocks (src/qpsubs.c:1578-1627): a new block at each chromosome change or once the
 * genetic position has moved blocklen morgans from the block's first SNP; SNPs with ignore
 * set get -1.  Returns the number of blocks. */
extern "C" int32_t gp_set_blocks(const int32_t *chrom, const double *gpos, const uint8_t *ignore,
                                 int64_t n, double blocklen, int32_t *tag)
{
  if (n < 0 || (n > 0 && (!chrom || !gpos))) return GP_ERR_ARG;
  int32_t nb = 0, lchrom = -1;
  int64_t xsize = 0;
  double fpos = -1.0e20;
  for (int64_t i = 0; i < n; ++i) {
    if (tag) tag[i] = -1;
    if (ignore && ignore[i]) continue;
    const double dis = gpos[i] - fpos;
    if (chrom[i] != lchrom || dis >= blocklen) {
      if (xsize > 0) ++nb;
      lchrom = chrom[i];
      fpos = gpos[i];
      xsize = 0;
    }
    if (tag) tag[i] = nb;
    ++xsize;
  }
  if (xsize > 0) ++nb;
  return nb;
}
