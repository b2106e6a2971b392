/*
 * FP64 products of the decoded genotype matrix with a dense FP64 panel.  The genotype
 * operand is never materialised: an element is T_s[code] where T_s is a 4-entry table of
 * the kept SNP s (code 3 = missing), decoded from the packed records per tile.
 *
 *   sum over SNPs    C[q][c]  = sum_s T_s[g(q,s)] B[s][c]   (sample scores fxvecs, the masked
 *                                                             normal equations of lsqproj)
 *   sum over samples C[s][c]  = sum_q T_s[g(q,s)] B[q][c]   (SNP weights ffvecs)
 *
 * These replace the scalar loops of smartpca.c:1485-1525 (ffvecs/fxvecs) and the per-sample
 * accumulation of regressit (src/regsubs.c:19-26).  64x64 output tiles, 16-deep k-steps,
 * 4x4 outputs per thread; the k range is split across grid.z when the output is small and
 * the partial results are summed in a fixed order.
 */
#include <cuda_runtime.h>

#include "gp_internal.h"
#include "gp_geno_gemm.h"

#define TT 64
#define TK 16

__device__ __forceinline__ uint32_t code_at(const uint8_t *__restrict__ rec, int32_t k)
{
  return (__ldg(rec + (k >> 2)) >> ((3 - (k & 3)) * 2)) & 3u;
}

__global__ void __launch_bounds__(256)
k_gemm_sum_snps(const uint8_t *__restrict__ geno, int64_t rlen, const int32_t *__restrict__ samp,
                const int32_t *__restrict__ spop, int32_t nsamp,
                const int32_t *__restrict__ snprec, const double *__restrict__ tab,
                const double *__restrict__ fill, int32_t npop, int32_t nsnp,
                const double *__restrict__ B, int64_t ldb, int32_t ncc, double *C, int64_t ldc,
                int32_t kper, int64_t split_stride)
{
  __shared__ double As[TK][TT + 1];
  __shared__ double Bs[TK][TT + 1];
  __shared__ double tabs[TK][4];
  __shared__ const uint8_t *recs[TK];
  __shared__ const double *fills[TK];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int32_t q0 = (int32_t)blockIdx.y * TT, c0 = (int32_t)blockIdx.x * TT;
  const int32_t kb = (int32_t)blockIdx.z * kper;
  const int32_t ke = kb + kper < nsnp ? kb + kper : nsnp;
  const int lk = tid & 15, lr = tid >> 4;
  int32_t srow[4], sp[4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    int32_t q = q0 + lr + 16 * p;
    srow[p] = q < nsamp ? samp[q] : -1;
    sp[p] = (fill && q < nsamp) ? spop[q] : -1;
  }
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

  for (int32_t k0 = kb; k0 < ke; k0 += TK) {
    if (tid < TK) {
      int32_t s = k0 + tid;
      if (s < ke) {
        recs[tid] = geno + (int64_t)snprec[s] * rlen;
        tabs[tid][0] = tab[4 * s];
        tabs[tid][1] = tab[4 * s + 1];
        tabs[tid][2] = tab[4 * s + 2];
        tabs[tid][3] = tab[4 * s + 3];
        fills[tid] = fill ? fill + (int64_t)s * npop : NULL;
      } else {
        recs[tid] = NULL;
      }
    }
    __syncthreads();
    const uint8_t *rec = recs[lk];
    const double *fl = fills[lk];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      double v = 0.0;
      if (rec && srow[p] >= 0) {
        const uint32_t cd = code_at(rec, srow[p]);
        v = (cd == 3u && fl && sp[p] >= 0) ? fl[sp[p]] : tabs[lk][cd];
      }
      As[lk][lr + 16 * p] = v;
    }
    /* B tile: 16 SNP rows x 64 columns */
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      int e = tid + 256 * p;
      int r = e >> 6, c = e & 63;
      int32_t s = k0 + r, cc = c0 + c;
      Bs[r][c] = (s < ke && cc < ncc) ? B[(int64_t)s * ldb + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        a[p] = As[k][ty + 16 * p];
        b[p] = Bs[k][tx + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[p][r] = fma(a[p], b[r], acc[p][r]);
    }
    __syncthreads();
  }
  double *o = C + (int64_t)blockIdx.z * split_stride;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    int32_t q = q0 + ty + 16 * p;
    if (q >= nsamp) continue;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int32_t c = c0 + tx + 16 * r;
      if (c < ncc) o[(int64_t)q * ldc + c] = acc[p][r];
    }
  }
}

__global__ void __launch_bounds__(256)
k_gemm_sum_samples(const uint8_t *__restrict__ geno, int64_t rlen,
                   const int32_t *__restrict__ samp, int32_t nsamp,
                   const int32_t *__restrict__ snprec, const double *__restrict__ tab,
                   int32_t nsnp, const double *__restrict__ B, int64_t ldb, int32_t ncc,
                   double *C, int64_t ldc, int32_t kper, int64_t split_stride)
{
  __shared__ double As[TK][TT + 1]; /* [sample][snp] */
  __shared__ double Bs[TK][TT + 1]; /* [sample][col] */
  __shared__ double tabs[TT][4];
  __shared__ const uint8_t *recs[TT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int32_t s0 = (int32_t)blockIdx.y * TT, c0 = (int32_t)blockIdx.x * TT;
  const int32_t kb = (int32_t)blockIdx.z * kper;
  const int32_t ke = kb + kper < nsamp ? kb + kper : nsamp;
  if (tid < TT) {
    int32_t s = s0 + tid;
    if (s < nsnp) {
      recs[tid] = geno + (int64_t)snprec[s] * rlen;
      tabs[tid][0] = tab[4 * s];
      tabs[tid][1] = tab[4 * s + 1];
      tabs[tid][2] = tab[4 * s + 2];
      tabs[tid][3] = tab[4 * s + 3];
    } else {
      recs[tid] = NULL;
    }
  }
  __syncthreads();
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  const int lk = tid & 15, lr = tid >> 4;
  for (int32_t k0 = kb; k0 < ke; k0 += TK) {
    int32_t q = k0 + lk;
    int32_t sidx = q < ke ? samp[q] : -1;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      int sl = lr + 16 * p;
      const uint8_t *rec = recs[sl];
      double v = 0.0;
      if (rec && sidx >= 0) v = tabs[sl][code_at(rec, sidx)];
      As[lk][sl] = v;
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      int e = tid + 256 * p;
      int r = e >> 6, c = e & 63;
      int32_t qq = k0 + r, cc = c0 + c;
      Bs[r][c] = (qq < ke && cc < ncc) ? B[(int64_t)qq * ldb + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        a[p] = As[k][ty + 16 * p];
        b[p] = Bs[k][tx + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[p][r] = fma(a[p], b[r], acc[p][r]);
    }
    __syncthreads();
  }
  double *o = C + (int64_t)blockIdx.z * split_stride;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    int32_t s = s0 + ty + 16 * p;
    if (s >= nsnp) continue;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int32_t c = c0 + tx + 16 * r;
      if (c < ncc) o[(int64_t)s * ldc + c] = acc[p][r];
    }
  }
}

__global__ void k_sum_parts(double *out, int64_t ldo, const double *part, int64_t ldp,
                            int64_t stride, int32_t nsplit, int32_t rows, int32_t cols)
{
  int64_t total = (int64_t)rows * cols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = idx / cols, c = idx - r * cols;
    double s = 0.0;
    for (int32_t t = 0; t < nsplit; ++t) s += part[t * stride + r * ldp + c];
    out[r * ldo + c] = s;
  }
}

static int pick_split(const gp_ctx *ctx, int64_t out_tiles, int32_t depth)
{
  int32_t nsplit = 1;
  if (out_tiles < 2 * ctx->num_sms) {
    nsplit = (int32_t)((2 * ctx->num_sms + out_tiles - 1) / out_tiles);
    int32_t maxsplit = (depth + 511) / 512;
    if (nsplit > maxsplit) nsplit = maxsplit;
    if (nsplit > 128) nsplit = 128;
    if (nsplit < 1) nsplit = 1;
  }
  return nsplit;
}

static int geno_gemm(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp,
                     const int32_t *d_spop, int32_t nsamp, const int32_t *d_snprec,
                     const double *d_tab, const double *d_fill, int32_t npop, int32_t nsnp,
                     const double *d_B, int64_t ldb, int32_t ncc, double *d_C, int64_t ldc)
{
  int32_t out_rows = sum_over_snps ? nsamp : nsnp;
  int32_t depth = sum_over_snps ? nsnp : nsamp;
  if (out_rows <= 0 || ncc <= 0) return GP_OK;
  if (depth <= 0) {
    GP_CUDA(ctx, cudaMemset2DAsync(d_C, (size_t)ldc * sizeof(double), 0,
                                   (size_t)ncc * sizeof(double), (size_t)out_rows, ctx->stream));
    return GP_OK;
  }
  int64_t tiles = (int64_t)((out_rows + TT - 1) / TT) * ((ncc + TT - 1) / TT);
  int32_t nsplit = pick_split(ctx, tiles, depth);
  int32_t kper = (depth + nsplit - 1) / nsplit;
  kper = (kper + TK - 1) / TK * TK;
  nsplit = (depth + kper - 1) / kper;
  dim3 grid((unsigned)((ncc + TT - 1) / TT), (unsigned)((out_rows + TT - 1) / TT),
            (unsigned)nsplit);
  double *dst = d_C;
  int64_t ld = ldc, stride = 0;
  if (nsplit > 1) {
    ld = ncc;
    stride = (int64_t)out_rows * ncc;
    int rc = gp_scratch2(ctx, sizeof(double) * (size_t)stride * nsplit, (void **)&dst);
    if (rc) return rc;
  }
  if (sum_over_snps)
    k_gemm_sum_snps<<<grid, 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, d_samp, d_spop,
                                                   nsamp, d_snprec, d_tab, d_fill, npop, nsnp,
                                                   d_B, ldb, ncc, dst, ld, kper, stride);
  else
    k_gemm_sum_samples<<<grid, 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, d_samp,
                                                      nsamp, d_snprec, d_tab, nsnp, d_B, ldb, ncc,
                                                      dst, ld, kper, stride);
  GP_LAUNCH_CHECK(ctx, "k_gemm_geno_f64");
  if (nsplit > 1) {
    int64_t total = (int64_t)out_rows * ncc;
    int blocks = (int)((total + 255) / 256);
    if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
    k_sum_parts<<<blocks, 256, 0, ctx->stream>>>(d_C, ldc, dst, ld, stride, nsplit, out_rows,
                                                 ncc);
    GP_LAUNCH_CHECK(ctx, "k_sum_parts");
  }
  return GP_OK;
}

int gp_geno_gemm_f64(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                     const int32_t *d_snprec, const double *d_tab, int32_t nsnp,
                     const double *d_B, int64_t ldb, int32_t ncc, double *d_C, int64_t ldc)
{
  return geno_gemm(ctx, sum_over_snps, d_samp, NULL, nsamp, d_snprec, d_tab, NULL, 0, nsnp, d_B,
                   ldb, ncc, d_C, ldc);
}

int gp_geno_gemm_f64_fill(gp_ctx *ctx, const int32_t *d_samp, const int32_t *d_spop,
                          int32_t nsamp, const int32_t *d_snprec, const double *d_tab,
                          const double *d_fill, int32_t npop, int32_t nsnp, const double *d_B,
                          int64_t ldb, int32_t ncc, double *d_C, int64_t ldc)
{
  return geno_gemm(ctx, 1, d_samp, d_spop, nsamp, d_snprec, d_tab, d_fill, npop, nsnp, d_B, ldb,
                   ncc, d_C, ldc);
}
