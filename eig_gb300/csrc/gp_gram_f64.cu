/*
 * Plain FP64 Gram (the drop-in precision): XTX[i][j] = sum over kept SNPs of v_i v_j for the
 * lower-triangle 64x64 tiles, replacing domult_increment_lookup / block_increment_binary
 * (src/eigensrc/smartpca.c:3361-3495) and domult_increment_normal (:3498-3561).
 *
 * The normalised values are never materialised: each k-step decodes a 64-row x 16-SNP tile
 * straight from the packed 2-bit records through the per-SNP value table (the 3-entry
 * tblock of the reference + 0 for missing).  The FP64 FMA pipe bounds this kernel (GB300's
 * FP64 rate is low by design); it is the parity baseline the split-BF16 path is measured
 * against.  When the triangle has fewer tiles than the GPU has SMs the SNP range is split
 * and the partial triangles are summed in a fixed order (deterministic).
 * With usepopsformissing (fill != NULL) a missing genotype of row i takes the value
 * fill[c*npop + rowpop[i]] of its population (0 for a row without one), the getcolxz values
 * of smartpca.c:3161-3184.
 */
#include <cuda_runtime.h>

#include "gp_internal.h"

#define GT 64   /* tile edge */
#define GK 16   /* SNPs per k-step */

__device__ __forceinline__ uint32_t geno_code(const uint8_t *__restrict__ rec, int32_t k)
{
  return (__ldg(rec + (k >> 2)) >> ((3 - (k & 3)) * 2)) & 3u;
}

/* tile pair index t -> (bi, bj) with bi >= bj, row-major over the lower triangle */
__device__ __forceinline__ void tri_index(int32_t t, int32_t *bi, int32_t *bj)
{
  int32_t i = (int32_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  while (i * (i + 1) / 2 > t) --i;
  *bi = i;
  *bj = t - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(256)
k_gram_f64(const uint8_t *__restrict__ geno, int64_t rlen, const int32_t *__restrict__ rows,
           int32_t nrows, const int32_t *__restrict__ cols, const int32_t *__restrict__ kept,
           int32_t nkept, const double *__restrict__ vtab, const double *__restrict__ fill,
           int32_t npop, const int32_t *__restrict__ rowpop, int32_t kper, double *out,
           int64_t ldo, int64_t split_stride)
{
  __shared__ double As[GK][GT + 1];
  __shared__ double Bs[GK][GT + 1];
  __shared__ double tabs[GK][4];
  __shared__ const uint8_t *recs[GK];
  __shared__ const double *fills[GK];

  int32_t bi, bj;
  tri_index((int32_t)blockIdx.x, &bi, &bj);
  const int32_t i0 = bi * GT, j0 = bj * GT;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;  /* 16x16 threads, 4x4 outputs each */
  const int32_t k_begin = (int32_t)blockIdx.y * kper;
  int32_t k_end = k_begin + kper;
  if (k_end > nkept) k_end = nkept;

  /* rows this thread decodes for the A and B tiles */
  const int lk = tid & 15, lr = tid >> 4;
  int32_t arow[4], brow[4], apop[4], bpop[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int32_t ri = i0 + lr + 16 * q, rj = j0 + lr + 16 * q;
    arow[q] = ri < nrows ? rows[ri] : -1;
    brow[q] = rj < nrows ? rows[rj] : -1;
    apop[q] = (fill && ri < nrows) ? rowpop[ri] : -1;
    bpop[q] = (fill && rj < nrows) ? rowpop[rj] : -1;
  }

  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

  for (int32_t k0 = k_begin; k0 < k_end; k0 += GK) {
    if (tid < GK) {
      int32_t kk = k0 + tid;
      if (kk < k_end) {
        int32_t c = kept[kk];
        recs[tid] = geno + (int64_t)cols[c] * rlen;
        tabs[tid][0] = vtab[4 * c];
        tabs[tid][1] = vtab[4 * c + 1];
        tabs[tid][2] = vtab[4 * c + 2];
        tabs[tid][3] = 0.0;
        fills[tid] = fill ? fill + (int64_t)c * npop : NULL;
      } else {
        recs[tid] = NULL;
      }
    }
    __syncthreads();
    const uint8_t *rec = recs[lk];
    const double *fl = fills[lk];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double va = 0.0, vb = 0.0;
      if (rec) {
        if (arow[q] >= 0) {
          const uint32_t cd = geno_code(rec, arow[q]);
          va = (cd == 3u && fl && apop[q] >= 0) ? fl[apop[q]] : tabs[lk][cd];
        }
        if (brow[q] >= 0) {
          const uint32_t cd = geno_code(rec, brow[q]);
          vb = (cd == 3u && fl && bpop[q] >= 0) ? fl[bpop[q]] : tabs[lk][cd];
        }
      }
      As[lk][lr + 16 * q] = va;
      Bs[lk][lr + 16 * q] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < GK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[k][ty + 16 * q];
        b[q] = Bs[k][tx + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
  double *o = out + (int64_t)blockIdx.y * split_stride;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    int32_t i = i0 + ty + 16 * p;
    if (i >= nrows) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int32_t j = j0 + tx + 16 * q;
      if (j < nrows && j <= i) o[(int64_t)i * ldo + j] = acc[p][q];
    }
  }
}

/* out[i] = sum over s of part[s*stride + i], fixed order, lower triangle only */
__global__ void k_reduce_splits(double *out, const double *part, int32_t nsplit, int64_t stride,
                                int32_t n, int64_t ldo)
{
  int64_t total = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = idx / n, j = idx - i * n;
    if (j > i) continue;
    double s = 0.0;
    for (int32_t t = 0; t < nsplit; ++t) s += part[t * stride + i * ldo + j];
    out[i * ldo + j] = s;
  }
}

/* copy the lower triangle to the upper one and sum the diagonal */
__global__ void k_symmetrize(double *x, int32_t n, double *trace_out)
{
  int64_t total = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = idx / n, j = idx - i * n;
    if (j > i) x[i * n + j] = x[j * n + i];
  }
  if (trace_out && blockIdx.x == 0) {
    __shared__ double red[256];
    double s = 0.0;
    for (int32_t i = threadIdx.x; i < n; i += blockDim.x) s += x[(int64_t)i * n + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) *trace_out = red[0];
  }
}

int gp_gram_fp64(gp_ctx *ctx)
{
  const int32_t n = ctx->nrows;
  const int32_t nt = (n + GT - 1) / GT;
  const int32_t ntiles = nt * (nt + 1) / 2;
  int32_t nsplit = 1;
  if (ctx->nkept > 0 && ntiles < 2 * ctx->num_sms) {
    nsplit = (2 * ctx->num_sms + ntiles - 1) / ntiles;
    int32_t maxsplit = (ctx->nkept + 255) / 256;
    if (nsplit > maxsplit) nsplit = maxsplit;
    if (nsplit > 64) nsplit = 64;
    if (nsplit < 1) nsplit = 1;
  }
  int32_t kper = (ctx->nkept + nsplit - 1) / nsplit;
  kper = (kper + GK - 1) / GK * GK;
  if (kper < GK) kper = GK;
  nsplit = ctx->nkept > 0 ? (ctx->nkept + kper - 1) / kper : 1;

  GP_CUDA(ctx, cudaMemsetAsync(ctx->d_xtx, 0, sizeof(double) * (size_t)n * n, ctx->stream));
  if (ctx->nkept == 0) return GP_OK;
  /* usepopsformissing: the filled values' table and the population fill values */
  const bool pf = ctx->npop > 0;
  const double *tab = pf ? ctx->d_gtab : ctx->d_vtab;
  const double *fill = pf ? ctx->d_gfill : NULL;
  const int32_t *rowpop = pf ? ctx->d_rowpop : NULL;
  if (nsplit == 1) {
    dim3 grid((unsigned)ntiles, 1);
    k_gram_f64<<<grid, 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, ctx->d_rows, n,
                                              ctx->d_cols, ctx->d_kept, ctx->nkept, tab, fill,
                                              ctx->npop, rowpop, kper, ctx->d_xtx, n, 0);
    GP_LAUNCH_CHECK(ctx, "k_gram_f64");
    ctx->gram_launches = 1;
    return GP_OK;
  }
  double *part;
  int64_t stride = (int64_t)n * n;
  int rc = gp_scratch(ctx, sizeof(double) * (size_t)stride * (size_t)nsplit, (void **)&part);
  if (rc) return rc;
  GP_CUDA(ctx, cudaMemsetAsync(part, 0, sizeof(double) * (size_t)stride * nsplit, ctx->stream));
  dim3 grid((unsigned)ntiles, (unsigned)nsplit);
  k_gram_f64<<<grid, 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, ctx->d_rows, n,
                                            ctx->d_cols, ctx->d_kept, ctx->nkept, tab, fill,
                                            ctx->npop, rowpop, kper, part, n, stride);
  GP_LAUNCH_CHECK(ctx, "k_gram_f64");
  ctx->gram_launches = 1;
  int blocks = (int)((stride + 255) / 256);
  if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
  k_reduce_splits<<<blocks, 256, 0, ctx->stream>>>(ctx->d_xtx, part, nsplit, stride, n, n);
  GP_LAUNCH_CHECK(ctx, "k_reduce_splits");
  return GP_OK;
}

int gp_launch_symmetrize_trace(gp_ctx *ctx, double *d_trace)
{
  int64_t total = (int64_t)ctx->nrows * ctx->nrows;
  int blocks = (int)((total + 255) / 256);
  if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
  if (blocks < 1) blocks = 1;
  k_symmetrize<<<blocks, 256, 0, ctx->stream>>>(ctx->d_xtx, ctx->nrows, d_trace);
  GP_LAUNCH_CHECK(ctx, "k_symmetrize");
  return GP_OK;
}
