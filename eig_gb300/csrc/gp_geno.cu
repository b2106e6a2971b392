/*
 * Genotype panel on the device: upload (packedancestrymap or PLINK .bed records), the
 * sample-selection bit mask, valid-genotype counts, and kernels (a)+(b): per-SNP allele and
 * missing counts with the kill rule and the normalised value table.
 *
 * Layout in HBM: one record of rlen_dev bytes per SNP (rlen_dev = ceil(N/4) rounded up to
 * 16 bytes), samples packed four per byte MSB first with the packedancestrymap code
 * (0/1/2 = count of the first allele, 3 = missing).  The selected rows are a 2-bit mask
 * word array in the same layout (0b11 under each selected sample), so a per-SNP count is
 * three popcounts per 16 samples: the SNP-major record is read once, coalesced, with no
 * gather.
 */
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "gp_internal.h"

/* ------------------------------------------------------------------------------------ */
/* BED -> packed recode: per byte, 4 samples LSB first, 00->2, 01->missing, 10->1, 11->0  */
/* (ancval src/mcio.c:3995-4009, bit order getbedgenos :3962-3966).                      */

__device__ __forceinline__ uint32_t bed_to_anc_code(uint32_t x)
{
  /* x: 2-bit bed code -> packed code (3 = missing) */
  return (x == 0u) ? 2u : (x == 1u) ? 3u : (x == 2u) ? 1u : 0u;
}

__global__ void k_recode_bed(uint8_t *rec, int64_t nsnp, int64_t rlen_dev, int64_t nbytes_used,
                             int32_t nind)
{
  int64_t total = nsnp * nbytes_used;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = i / nbytes_used, b = i - s * nbytes_used;
    uint8_t *p = rec + s * rlen_dev + b;
    uint32_t in = *p, out = 0;
    for (int t = 0; t < 4; ++t) {
      int64_t k = b * 4 + t;
      uint32_t code = (k < nind) ? bed_to_anc_code((in >> (2 * t)) & 3u) : 3u;
      out |= code << ((3 - t) * 2);
    }
    *p = (uint8_t)out;
  }
}

/* records of src_pitch bytes (used of them genotype bytes) into the 16-byte device pitch,
 * one 16-byte chunk per thread; bytes past used read as 0xFF (missing) */
__global__ void k_repitch(const uint8_t *__restrict__ src, int64_t src_pitch, int64_t used,
                          uint8_t *__restrict__ dst, int64_t rlen_dev, int64_t nsnp)
{
  const int64_t chunks = rlen_dev >> 4, total = nsnp * chunks;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = i / chunks, j = i - s * chunks, b0 = 16 * j;
    const uint8_t *p = src + s * src_pitch + b0;
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t v = 0;
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int64_t b = b0 + 4 * q + t;
        const uint32_t by = b < used ? (uint32_t)p[4 * q + t] : 0xFFu;
        v |= by << (8 * t);
      }
      w[q] = v;
    }
    *(uint4 *)(dst + s * rlen_dev + b0) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

/* set the bytes after the last sample of each record to 0xFF (missing) */
__global__ void k_pad_records(uint8_t *rec, int64_t nsnp, int64_t rlen_dev, int32_t nind)
{
  int64_t first = nind >> 2;          /* byte holding sample nind (partial) */
  int64_t npad = rlen_dev - first;
  int64_t total = nsnp * npad;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = i / npad, b = first + (i - s * npad);
    uint8_t *p = rec + s * rlen_dev + b;
    uint32_t v = *p;
    for (int t = 0; t < 4; ++t) {
      int64_t k = b * 4 + t;
      if (k >= nind) v |= 3u << ((3 - t) * 2);
    }
    *p = (uint8_t)v;
  }
}

__global__ void k_set_missing(uint8_t *rec, int64_t rlen_dev, const int64_t *pairs, int64_t n,
                              int64_t nsnp, int32_t nind)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = pairs[2 * i], k = pairs[2 * i + 1];
    if (s < 0 || s >= nsnp || k < 0 || k >= nind) continue;
    uint32_t *w = (uint32_t *)(rec + s * rlen_dev + ((k >> 2) & ~3LL));
    uint32_t shift = (uint32_t)((k & 15) >> 2) * 8u + (3u - (uint32_t)(k & 3)) * 2u;
    atomicOr(w, 3u << shift);
  }
}

static int grid_for(const gp_ctx *ctx, int64_t work, int threads)
{
  int64_t g = (work + threads - 1) / threads;
  int64_t cap = (int64_t)ctx->num_sms * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

extern "C" int gp_load_genotypes(gp_ctx *ctx, const uint8_t *records, int64_t record_bytes,
                                 int64_t nsnp, int32_t nind, int32_t code)
{
  if (!ctx) return GP_ERR_ARG;
  if (!records || nsnp <= 0 || nind <= 0 || (code != GP_CODE_PACKED && code != GP_CODE_BED))
    return gp_fail(ctx, GP_ERR_ARG, "gp_load_genotypes: bad arguments");
  int64_t used = ((int64_t)nind + 3) / 4;
  if (record_bytes < used)
    return gp_fail(ctx, GP_ERR_ARG, "gp_load_genotypes: record_bytes %lld < ceil(N/4) %lld",
                   (long long)record_bytes, (long long)used);
  int64_t rlen_dev = (used + 15) / 16 * 16;
  size_t bytes = (size_t)(rlen_dev * nsnp);
  /* the panel's allocation is kept while it is large enough (no cudaFree / cudaMalloc, and
   * their synchronisation, when a handle reloads panels of the same size) */
  if (ctx->d_geno && bytes > ctx->geno_cap) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_geno);
    ctx->d_geno = NULL;
    ctx->geno_cap = 0;
  }
  if (!ctx->d_geno) {
    cudaError_t e = cudaMalloc((void **)&ctx->d_geno, bytes);
    if (e != cudaSuccess) {
      ctx->d_geno = NULL;
      return gp_fail(ctx, GP_ERR_NOMEM, "gp_load_genotypes: cudaMalloc %zu bytes: %s", bytes,
                     cudaGetErrorString(e));
    }
    ctx->geno_cap = bytes;
  }
  ctx->nsnp_all = nsnp;
  ctx->nind_all = nind;
  ctx->rlen_dev = rlen_dev;
  ctx->nrows = ctx->ncols = 0;
  ctx->codes4_rows = 0;
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  /* one contiguous host-to-device copy (a pitched copy of many short rows is slow), then
   * the records are re-pitched on the device when the host pitch differs */
  const size_t hbytes = (size_t)record_bytes * (size_t)nsnp;
  if (record_bytes == rlen_dev) {
    GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_geno, records, hbytes, cudaMemcpyHostToDevice,
                           ctx->stream));
  } else {
    uint8_t *stage;
    int rc = gp_scratch2(ctx, hbytes + 16, (void **)&stage);
    if (rc) return rc;
    GP_CUDA(ctx, gp_memcpy(ctx, stage, records, hbytes, cudaMemcpyHostToDevice, ctx->stream));
    k_repitch<<<grid_for(ctx, nsnp * (rlen_dev >> 4), 256), 256, 0, ctx->stream>>>(
        stage, record_bytes, used, ctx->d_geno, rlen_dev, nsnp);
    GP_LAUNCH_CHECK(ctx, "k_repitch");
  }
  if (code == GP_CODE_BED) {
    k_recode_bed<<<grid_for(ctx, nsnp * used, 256), 256, 0, ctx->stream>>>(
        ctx->d_geno, nsnp, rlen_dev, used, nind);
    GP_LAUNCH_CHECK(ctx, "k_recode_bed");
  }
  k_pad_records<<<grid_for(ctx, nsnp * (rlen_dev - (nind >> 2)), 256), 256, 0, ctx->stream>>>(
      ctx->d_geno, nsnp, rlen_dev, nind);
  GP_LAUNCH_CHECK(ctx, "k_pad_records");
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GP_OK;
}

extern "C" int gp_genotype_shape(const gp_ctx *ctx, int64_t *nsnp, int32_t *nind)
{
  if (!ctx) return GP_ERR_ARG;
  if (nsnp) *nsnp = ctx->d_geno ? ctx->nsnp_all : 0;
  if (nind) *nind = ctx->d_geno ? ctx->nind_all : 0;
  return GP_OK;
}

extern "C" int gp_set_missing(gp_ctx *ctx, const int64_t *pairs, int64_t npairs)
{
  if (!ctx) return GP_ERR_ARG;
  if (!ctx->d_geno) return gp_fail(ctx, GP_ERR_STATE, "gp_set_missing: no genotypes loaded");
  if (npairs <= 0) return GP_OK;
  if (!pairs) return gp_fail(ctx, GP_ERR_ARG, "gp_set_missing: pairs is NULL");
  int64_t *d_pairs;
  int rc = gp_scratch(ctx, sizeof(int64_t) * 2 * (size_t)npairs, (void **)&d_pairs);
  if (rc) return rc;
  GP_CUDA(ctx, gp_memcpy(ctx, d_pairs, pairs, sizeof(int64_t) * 2 * (size_t)npairs,
                               cudaMemcpyHostToDevice, ctx->stream));
  k_set_missing<<<grid_for(ctx, npairs, 256), 256, 0, ctx->stream>>>(
      ctx->d_geno, ctx->rlen_dev, d_pairs, npairs, ctx->nsnp_all, ctx->nind_all);
  GP_LAUNCH_CHECK(ctx, "k_set_missing");
  ctx->codes4_rows = 0;
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GP_OK;
}

/*
 * missingmode: every genotype of a real sample becomes the indicator of being observed,
 * 1 when its code is 0/1/2 and 0 when it is missing (setmiss src/qpsubs.c:462-483); the pad
 * codes past the last sample stay missing.  One 32-bit word (16 codes) per thread.
 */
__global__ void k_missingmode(uint8_t *geno, int64_t rlen_dev, int64_t nsnp, int32_t nind)
{
  const int64_t wpr = rlen_dev >> 2, total = nsnp * wpr;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = i % wpr;
    uint32_t *pw = (uint32_t *)geno + i;
    const uint32_t x = *pw;
    /* per 2-bit code (h, l): missing = h & l; observed -> 01, missing -> 00 */
    const uint32_t miss = (x >> 1) & x & 0x55555555u;
    uint32_t y = ~miss & 0x55555555u;
    /* codes of sample k sit in byte k>>2 (little-endian word w holds samples 16w..16w+15) */
    const int64_t k0 = w * 16;
    if (k0 + 16 > nind) {
      uint32_t keep = 0;
      for (int j = 0; j < 16; ++j)
        if (k0 + j < nind) keep |= 3u << ((uint32_t)(j >> 2) * 8u + (3u - (uint32_t)(j & 3)) * 2u);
      y = (y & keep) | (x & ~keep);
    }
    *pw = y;
  }
}

extern "C" int gp_set_missingmode(gp_ctx *ctx)
{
  if (!ctx) return GP_ERR_ARG;
  if (!ctx->d_geno) return gp_fail(ctx, GP_ERR_STATE, "gp_set_missingmode: no genotypes loaded");
  const int64_t words = ctx->nsnp_all * (ctx->rlen_dev >> 2);
  k_missingmode<<<grid_for(ctx, words, 256), 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev,
                                                                   ctx->nsnp_all, ctx->nind_all);
  GP_LAUNCH_CHECK(ctx, "k_missingmode");
  ctx->codes4_rows = 0;
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */
/* selection masks                                                                        */

__global__ void k_rowmask_from_list(uint32_t *mask, int64_t nwords, const int32_t *rows,
                                    int32_t nrows)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t k = rows[i];
    /* byte k>>2, bits (3-(k&3))*2 ; little-endian word w = k>>4 holds bytes 4w..4w+3 */
    uint32_t shift = (uint32_t)((k & 15) >> 2) * 8u + (3u - (uint32_t)(k & 3)) * 2u;
    atomicOr(&mask[k >> 4], 3u << shift);
  }
}

__global__ void k_rowmask_from_flags(uint32_t *mask, int64_t nwords, const uint8_t *use,
                                     int32_t nind)
{
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nwords;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    for (int j = 0; j < 16; ++j) {
      int64_t k = w * 16 + j;
      if (k < nind && use[k]) m |= 3u << ((uint32_t)(j >> 2) * 8u + (3u - (uint32_t)(j & 3)) * 2u);
    }
    mask[w] = m;
  }
}

extern "C" int gp_set_samples(gp_ctx *ctx, const int32_t *xindex, int32_t nrows)
{
  if (!ctx) return GP_ERR_ARG;
  if (!ctx->d_geno) return gp_fail(ctx, GP_ERR_STATE, "gp_set_samples: no genotypes loaded");
  if (nrows < 1 || nrows > ctx->nind_all || !xindex)
    return gp_fail(ctx, GP_ERR_ARG, "gp_set_samples: nrows %d out of range", nrows);
  for (int32_t i = 0; i < nrows; ++i) {
    if (xindex[i] < 0 || xindex[i] >= ctx->nind_all || (i > 0 && xindex[i] <= xindex[i - 1]))
      return gp_fail(ctx, GP_ERR_ARG, "gp_set_samples: xindex must be ascending in [0,N)");
  }
  int rc = gp_realloc(ctx, (void **)&ctx->d_rows, sizeof(int32_t) * (size_t)ctx->nind_all);
  if (rc) return rc;
  int64_t nwords = ctx->rlen_dev / 4;
  rc = gp_realloc(ctx, (void **)&ctx->d_rowmask, sizeof(uint32_t) * (size_t)nwords);
  if (rc) return rc;
  GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_rows, xindex, sizeof(int32_t) * (size_t)nrows,
                               cudaMemcpyHostToDevice, ctx->stream));
  GP_CUDA(ctx, cudaMemsetAsync(ctx->d_rowmask, 0, sizeof(uint32_t) * (size_t)nwords,
                               ctx->stream));
  k_rowmask_from_list<<<grid_for(ctx, nrows, 256), 256, 0, ctx->stream>>>(
      ctx->d_rowmask, nwords, ctx->d_rows, nrows);
  GP_LAUNCH_CHECK(ctx, "k_rowmask_from_list");
  int32_t *hr = (int32_t *)realloc(ctx->h_rows, sizeof(int32_t) * (size_t)nrows);
  if (!hr) return gp_fail(ctx, GP_ERR_NOMEM, "gp_set_samples: host row list");
  memcpy(hr, xindex, sizeof(int32_t) * (size_t)nrows);
  ctx->h_rows = hr;
  ctx->nrows = nrows;
  ctx->npop = 0; /* the row populations belong to the previous rows */
  ctx->codes4_rows = 0;
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GP_OK;
}

extern "C" int gp_set_snps(gp_ctx *ctx, const int32_t *snp_index, int32_t ncols)
{
  if (!ctx) return GP_ERR_ARG;
  if (!ctx->d_geno) return gp_fail(ctx, GP_ERR_STATE, "gp_set_snps: no genotypes loaded");
  if (ncols < 1 || (int64_t)ncols > ctx->nsnp_all || !snp_index)
    return gp_fail(ctx, GP_ERR_ARG, "gp_set_snps: ncols %d out of range", ncols);
  for (int32_t i = 0; i < ncols; ++i)
    if (snp_index[i] < 0 || (int64_t)snp_index[i] >= ctx->nsnp_all)
      return gp_fail(ctx, GP_ERR_ARG, "gp_set_snps: snp index %d out of range", snp_index[i]);
  int rc = gp_realloc(ctx, (void **)&ctx->d_cols, sizeof(int32_t) * (size_t)ncols);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_cnt, sizeof(int32_t) * 3 * (size_t)ncols);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_killed, (size_t)ncols);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_vtab, sizeof(double) * 4 * (size_t)ncols);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_xmean, sizeof(double) * (size_t)ncols);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_xfancy, sizeof(double) * (size_t)ncols);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_kept, sizeof(int32_t) * (size_t)ncols);
  if (rc) return rc;
  GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_cols, snp_index, sizeof(int32_t) * (size_t)ncols,
                               cudaMemcpyHostToDevice, ctx->stream));
  ctx->ncols = ncols;
  ctx->codes4_rows = 0;
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */
/* valid-genotype counts                                                                  */

/* per SNP: number of non-missing genotypes among the samples of `mask` (one warp / SNP) */
__global__ void k_snp_valid(const uint8_t *geno, int64_t rlen_dev, int64_t nsnp,
                            const uint32_t *mask, const uint8_t *snp_use, int32_t *out)
{
  /* 16-byte words (rlen_dev and the mask are 16-byte aligned) */
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int64_t nw = (int64_t)gridDim.x * blockDim.x >> 5;
  int64_t words4 = rlen_dev >> 4;
  const uint4 *m4 = (const uint4 *)mask;
  for (int64_t s = warp; s < nsnp; s += nw) {
    if (snp_use && !snp_use[s]) {
      if (lane == 0) out[s] = 0;
      continue;
    }
    const uint4 *rec = (const uint4 *)(geno + s * rlen_dev);
    int32_t cnt = 0;
    for (int64_t i = lane; i < words4; i += 32) {
      const uint4 w = __ldg(rec + i), m = __ldg(m4 + i);
      const uint32_t wv[4] = {w.x, w.y, w.z, w.w}, mv[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t sel = mv[q] & 0x55555555u;
        const uint32_t miss = (wv[q] >> 1) & wv[q] & 0x55555555u;
        cnt += __popc(sel) - __popc(miss & sel);
      }
    }
    for (int o = 16; o; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if (lane == 0) out[s] = cnt;
  }
}

/* per sample: number of non-missing genotypes over the used SNPs.  Thread = one word of
 * 16 samples, looping over a slice of SNPs eight records at a time (loads first; an unused
 * SNP reads as all-missing); the observed bits are summed in 4-bit fields of two words
 * (fields 0, 2, .. and 1, 3, ..), flushed into per-sample counts every 15 SNPs; partial
 * counts are summed with atomics. */
__global__ void k_sample_valid(const uint8_t *geno, int64_t rlen_dev, int64_t nsnp,
                               const uint8_t *snp_use, int32_t nind, int32_t *out,
                               int64_t snps_per_slice)
{
  int64_t words = rlen_dev >> 2;
  int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (w >= words) return;
  int64_t s0 = (int64_t)blockIdx.y * snps_per_slice;
  int64_t s1 = s0 + snps_per_slice < nsnp ? s0 + snps_per_slice : nsnp;
  int32_t cnt[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) cnt[j] = 0;
  uint32_t acc_a = 0, acc_b = 0;
  int pend = 0;
  auto flush = [&]() {
#pragma unroll
    for (int f = 0; f < 16; ++f) {
      /* field f (bits 2f, 2f+1) is sample (f >> 2) * 4 + 3 - (f & 3) of the word */
      const uint32_t v = ((f & 1) ? acc_b : acc_a) >> (4 * (f >> 1));
      cnt[(f >> 2) * 4 + 3 - (f & 3)] += (int32_t)(v & 0xFu);
    }
    acc_a = acc_b = 0;
    pend = 0;
  };
  const uint32_t *col = (const uint32_t *)geno + w;
  const int64_t stride = rlen_dev >> 2;
  for (int64_t s = s0; s < s1; s += 8) {
    uint32_t v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int64_t su = s + u;
      v[u] = su < s1 ? __ldg(col + su * stride) : 0xFFFFFFFFu;
      if (snp_use && su < s1 && !snp_use[su]) v[u] = 0xFFFFFFFFu;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint32_t ok = ~((v[u] >> 1) & v[u]) & 0x55555555u;
      acc_a += ok & 0x11111111u;
      acc_b += (ok >> 2) & 0x11111111u;
      if (++pend == 15) flush();
    }
  }
  flush();
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    int64_t k = w * 16 + j;
    if (k < nind && cnt[j]) atomicAdd(&out[k], cnt[j]);
  }
}

extern "C" int gp_valid_counts(gp_ctx *ctx, const uint8_t *sample_use, const uint8_t *snp_use,
                               int32_t *snp_valid, int32_t *sample_valid)
{
  if (!ctx) return GP_ERR_ARG;
  if (!ctx->d_geno) return gp_fail(ctx, GP_ERR_STATE, "gp_valid_counts: no genotypes loaded");
  int64_t nsnp = ctx->nsnp_all, nwords = ctx->rlen_dev / 4;
  size_t need = (size_t)nsnp + (size_t)ctx->nind_all + sizeof(uint32_t) * (size_t)nwords +
                sizeof(int32_t) * ((size_t)nsnp + (size_t)ctx->nind_all) + 64;
  uint8_t *base;
  int rc = gp_scratch(ctx, need, (void **)&base);
  if (rc) return rc;
  /* the mask first: 16-byte aligned for k_snp_valid's vector loads */
  uint32_t *d_mask = (uint32_t *)base;
  int32_t *d_sv = (int32_t *)(d_mask + nwords);
  int32_t *d_iv = d_sv + nsnp;
  uint8_t *d_su = (uint8_t *)(d_iv + ctx->nind_all);
  uint8_t *d_pu = d_su + nsnp;
  if (snp_use)
    GP_CUDA(ctx, gp_memcpy(ctx, d_su, snp_use, (size_t)nsnp, cudaMemcpyHostToDevice,
                                 ctx->stream));
  if (sample_use) {
    GP_CUDA(ctx, gp_memcpy(ctx, d_pu, sample_use, (size_t)ctx->nind_all,
                                 cudaMemcpyHostToDevice, ctx->stream));
  } else {
    GP_CUDA(ctx, cudaMemsetAsync(d_pu, 1, (size_t)ctx->nind_all, ctx->stream));
  }
  k_rowmask_from_flags<<<grid_for(ctx, nwords, 256), 256, 0, ctx->stream>>>(d_mask, nwords, d_pu,
                                                                           ctx->nind_all);
  GP_LAUNCH_CHECK(ctx, "k_rowmask_from_flags");
  if (snp_valid) {
    k_snp_valid<<<grid_for(ctx, nsnp * 32, 256), 256, 0, ctx->stream>>>(
        ctx->d_geno, ctx->rlen_dev, nsnp, d_mask, NULL, d_sv);
    GP_LAUNCH_CHECK(ctx, "k_snp_valid");
    GP_CUDA(ctx, gp_memcpy(ctx, snp_valid, d_sv, sizeof(int32_t) * (size_t)nsnp,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (sample_valid) {
    GP_CUDA(ctx, cudaMemsetAsync(d_iv, 0, sizeof(int32_t) * (size_t)ctx->nind_all, ctx->stream));
    int64_t slice = 4096;
    dim3 grid((unsigned)((nwords + 127) / 128), (unsigned)((nsnp + slice - 1) / slice));
    k_sample_valid<<<grid, 128, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, nsnp,
                                                  snp_use ? d_su : NULL, ctx->nind_all, d_iv,
                                                  slice);
    GP_LAUNCH_CHECK(ctx, "k_sample_valid");
    GP_CUDA(ctx, gp_memcpy(ctx, sample_valid, d_iv, sizeof(int32_t) * (size_t)ctx->nind_all,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  }
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */
/* kernels (a)+(b): per-SNP counts, kill rule, normalised value table                     */

/*
 * A warp per group of 32 selected columns.  For each column of the group the warp's lanes
 * stream its record (16-byte loads) and count n0 = sum g and nmiss over the selected rows; the
 * butterfly reduction leaves the totals in every lane and lane j keeps column j's.  (Four
 * columns at a time with ten loads in flight per lane measured slower: 116 against 86 us on
 * a 5,000 x 200,000 panel, at 60 registers against 40 and fewer resident warps.)  n1 = 2(n-nmiss) - n0 equals the reference's sum (2-g) over the same rows
 * (getcolxz_binary1 smartpca.c:3270-3279).  Then every lane restates fvadjust_binary
 * (:2282-2313) for its own column with the same IEEE double operations in the same order (no
 * contraction), so the table is bit-identical to the reference's tblock entries.  The FP64
 * epilogue thus runs on all 32 lanes at once: GB300 issues FP64 instructions at a small
 * fraction of the FP32 rate, and one lane per warp doing it left the kernel FP64-issue bound.
 */
__global__ void __launch_bounds__(256)
k_snp_stats(const uint8_t *__restrict__ geno, int64_t rlen_dev,
            const uint32_t *__restrict__ rowmask, const int32_t *__restrict__ cols,
            int32_t ncols, int32_t nrows, gp_xtx_opts o, int32_t *cnt,
            uint8_t *killed, double *vtab, double *xmean, double *xfancy)
{
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  /* 16-byte words (rlen_dev and the row mask are 16-byte aligned) */
  const int64_t words4 = rlen_dev >> 4;
  const uint4 *m4 = (const uint4 *)rowmask;
  const int64_t ngroups = ((int64_t)ncols + 31) >> 5;
  for (int64_t g = warp; g < ngroups; g += nw) {
    const int64_t c_first = g << 5;
    const int ncg = (int)((int64_t)ncols - c_first < 32 ? (int64_t)ncols - c_first : 32);
    int32_t my_sumg = 0, my_nmiss = 0;
#pragma unroll 2
    for (int j = 0; j < ncg; ++j) {
      const uint4 *rec = (const uint4 *)(geno + (int64_t)cols[c_first + j] * rlen_dev);
      int32_t sumg = 0, nmiss = 0;
      for (int64_t i = lane; i < words4; i += 32) {
        const uint4 w4 = __ldg(rec + i), s4 = __ldg(m4 + i);
        const uint32_t wv[4] = {w4.x, w4.y, w4.z, w4.w}, sv[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t w = wv[q], sel = sv[q] & 0x55555555u;
          const uint32_t hi = (w >> 1) & 0x55555555u, lo = w & 0x55555555u;
          const uint32_t miss = hi & lo & sel;
          const uint32_t obs = sel & ~miss;
          sumg += 2 * __popc(hi & obs) + __popc(lo & obs);
          nmiss += __popc(miss);
        }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        sumg += __shfl_xor_sync(0xffffffffu, sumg, off);
        nmiss += __shfl_xor_sync(0xffffffffu, nmiss, off);
      }
      if (lane == j) {
        my_sumg = sumg;
        my_nmiss = nmiss;
      }
    }
    if (lane < ncg) {
      const int64_t c = c_first + lane;
      const int32_t nmiss = my_nmiss;
      int32_t c0 = my_sumg, c1 = 2 * (nrows - nmiss) - my_sumg;
      double v0 = 0.0, v1 = 0.0, v2 = 0.0, pm = 0.0, yf = 0.0;
      int kill;
      if (nrows == nmiss) {
        /* fvadjust_binary returns -999: xmean = xfancy = 0, n0 = n1 = -1, killed */
        c0 = c1 = -1;
        kill = 1;
      } else {
        double ynum = (double)(nrows - nmiss);
        double ysum = (double)c0;
        double ymean = __ddiv_rn(ysum, ynum);
        double yfancy = 1.0;
        if (o.fancynorm) {
          double p = __dmul_rn(0.5, ymean);
          if (o.altnormstyle == 0) p = __ddiv_rn(__dadd_rn(ysum, 1.0), __dadd_rn(__dmul_rn(2.0, ynum), 2.0));
          double y = __dmul_rn(p, __dsub_rn(1.0, p));
          if (y > 0.0) yfancy = __ddiv_rn(1.0, __dsqrt_rn(y));
        }
        v0 = __dmul_rn(-ymean, yfancy);
        v1 = __dmul_rn(__dsub_rn(1.0, ymean), yfancy);
        v2 = __dmul_rn(__dsub_rn(2.0, ymean), yfancy);
        pm = __dmul_rn(ymean, yfancy);
        yf = yfancy;
        int32_t t = c0 < c1 ? c0 : c1;
        kill = (t < o.minallelecnt) || (nmiss > o.maxmissing) || (t == 0);
      }
      cnt[3 * c] = c0;
      cnt[3 * c + 1] = c1;
      cnt[3 * c + 2] = nmiss;
      killed[c] = (uint8_t)kill;
      xmean[c] = pm;
      xfancy[c] = yf;
      double *vt = vtab + 4 * c;
      if (kill) {
        vt[0] = vt[1] = vt[2] = vt[3] = 0.0;
      } else {
        vt[0] = v0;
        vt[1] = v1;
        vt[2] = v2;
        vt[3] = 0.0;
      }
    }
  }
}

int gp_launch_snp_stats(gp_ctx *ctx, const gp_xtx_opts *o)
{
  int64_t threads = ((int64_t)ctx->ncols + 31) / 32 * 32;  /* a warp per 32 columns */
  GP_CUDA(ctx, cudaEventRecord(ctx->ev_c0, ctx->stream));
  k_snp_stats<<<grid_for(ctx, threads, 256), 256, 0, ctx->stream>>>(
      ctx->d_geno, ctx->rlen_dev, ctx->d_rowmask, ctx->d_cols, ctx->ncols, ctx->nrows, *o,
      ctx->d_cnt, ctx->d_killed, ctx->d_vtab, ctx->d_xmean, ctx->d_xfancy);
  GP_LAUNCH_CHECK(ctx, "k_snp_stats");
  GP_CUDA(ctx, cudaEventRecord(ctx->ev_c1, ctx->stream));
  /* one read of each selected record and the row mask, 61 bytes out per column */
  ctx->counts_bytes = (int64_t)ctx->ncols * (ctx->rlen_dev + 61) + ctx->rlen_dev;
  return GP_OK;
}
