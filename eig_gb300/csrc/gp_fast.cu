/*
 * fastmode: randomized block-Krylov PCA (kjg_fpca src/ksrc/kjg_fpca.c:24-102, data table of
 * setgval src/gval.c:31-87).
 *
 *   X (M SNPs x N samples), X[s][i] = ((g - mean_s) fancy_s)/sqrt(2), missing -> 0
 *   G_0 = Omega (N x L);  for i < I:  Q_i = X G_i,  G_{i+1} = X^T Q_i / M;  Q_I = X G_I
 *   Q = [Q_0 .. Q_I]  (M x (I+1)L)  ->  orthonormal basis of its columns
 *   B = X^T Q  (N x (I+1)L);  top K left singular vectors of B and S^2/M
 *
 * Products with X use the exact sliced tensor-core products (gp_geno_tc.cu) for the split
 * precisions, written as X = (G fancy - O xmean)/sqrt(2) with G the allele counts and O the
 * observed mask (the FP64 SIMT products with the value table for GP_PREC_FP64).  The code
 * operands are built once per call; with every sample selected the SNP-major device records
 * themselves are the operand of X G.  The orthonormal basis comes from FP64 Householder QR
 * (cuSOLVER geqrf/orgqr: the reference takes the left singular vectors of an SVD, any
 * orthonormal basis of the same column space gives the same B's singular triplets), and the
 * SVD of B from the eigen-decomposition of the small Gram B^T B (cuBLAS DGEMM + cuSOLVER syevd,
 * FP64): U_K = B V_K / S_K, eval = S^2 / M.
 */
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <math.h>
#include <stdlib.h>

#include "gp_geno_gemm.h"
#include "gp_geno_tc.h"
#include "gp_internal.h"

static const double INV_SQRT2 = 0.70710678118654752440;

/* Omega (N x L row-major): polar Box-Muller pairs from a seeded splitmix stream; with an odd
 * L the last column holds uniform draws, as kjg_gsl_ran_ugaussian_matrix does
 * (src/ksrc/kjg_gsl.c:167-190) */
static void make_omega(uint64_t seed, int32_t n, int32_t L, double *om)
{
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
  auto uni = [&st]() {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  for (int32_t i = 0; i < n; ++i) {
    double *row = om + (size_t)i * L;
    int32_t j = 0;
    for (; j + 1 < L; j += 2) {
      double x, y, r2;
      do {
        x = -1.0 + 2.0 * uni();
        y = -1.0 + 2.0 * uni();
        r2 = x * x + y * y;
      } while (r2 > 1.0 || r2 == 0.0);
      double f = sqrt(-2.0 * log(r2) / r2);
      row[j] = x * f;
      row[j + 1] = y * f;
    }
    if (j < L) row[j] = uni();
  }
}

/* Q(:, col0 + j) [column-major, ldq] = (fancy_s Yg[s][j] - xmean_s Yo[s][j]) / sqrt2 */
__global__ void k_fast_combine_xg(double *Q, int64_t ldq, int32_t col0, const double *yg,
                                  const double *yo, const int32_t *kept, const double *xfancy,
                                  const double *xmean, int32_t nk, int32_t L, double scale)
{
  int64_t total = (int64_t)nk * L;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = idx / L;
    int32_t j = (int32_t)(idx - s * L);
    int32_t c = kept[s];
    Q[(int64_t)(col0 + j) * ldq + s] = (xfancy[c] * yg[idx] - xmean[c] * yo[idx]) * scale;
  }
}

/* panels for X^T Q: a[s][j] = fancy_s Q[s][j] / sqrt2, b[s][j] = xmean_s Q[s][j] / sqrt2 */
__global__ void k_fast_panels(double *a, double *b, const double *Q, int64_t ldq, int32_t c0,
                              int32_t ncols, const int32_t *kept, const double *xfancy,
                              const double *xmean, int32_t nk)
{
  int64_t total = (int64_t)nk * ncols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = idx / ncols;
    int32_t j = (int32_t)(idx - s * ncols);
    int32_t c = kept[s];
    double q = Q[(int64_t)(c0 + j) * ldq + s] * INV_SQRT2;
    a[idx] = xfancy[c] * q;
    b[idx] = xmean[c] * q;
  }
}

/* Q(:, col0 + j) [column-major, ldq] = Y[s][j] (FP64 path: the table already holds X) */
__global__ void k_fast_scatter(double *Q, int64_t ldq, int32_t col0, const double *Y, int32_t nk,
                               int32_t L)
{
  int64_t total = (int64_t)nk * L;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = idx / L;
    int32_t j = (int32_t)(idx - s * L);
    Q[(int64_t)(col0 + j) * ldq + s] = Y[idx];
  }
}

/* P[s][j] (row-major, ncols) = Q(s, c0 + j) */
__global__ void k_fast_gather(double *P, const double *Q, int64_t ldq, int32_t c0, int32_t ncols,
                              int32_t nk)
{
  int64_t total = (int64_t)nk * ncols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = idx / ncols;
    int32_t j = (int32_t)(idx - s * ncols);
    P[idx] = Q[(int64_t)(c0 + j) * ldq + s];
  }
}

/* vtab scaled by 1/sqrt2 for the FP64 products, per kept column */
__global__ void k_fast_vtab(const int32_t *kept, int32_t nk, const int32_t *cols, const double *vtab,
                            int32_t *snprec, double *vt)
{
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
    int32_t c = kept[k];
    snprec[k] = cols[c];
    for (int t = 0; t < 4; ++t) vt[4 * k + t] = vtab[4 * c + t] * INV_SQRT2;
  }
}

/* row-major [n][L] <- scale * row-major src (the next power-iteration block) */
__global__ void k_scale_copy(double *dst, const double *src, int64_t n, double scale)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] * scale;
}

/* evec[j][i] = (B V)[i][col_j] / sigma_j for the top K (V columns ascending in syevd) */
__global__ void k_fast_evecs(double *evecs, const double *BV, int32_t n, int32_t c4, int32_t K,
                             const double *w)
{
  int64_t total = (int64_t)n * K;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int32_t j = (int32_t)(idx / n);
    int64_t i = idx - (int64_t)j * n;
    int32_t col = c4 - 1 - j;
    double sig = sqrt(fmax(w[col], 0.0));
    evecs[idx] = sig > 0.0 ? BV[(int64_t)col * n + i] / sig : 0.0;
  }
}

static int grid_for_fast(const gp_ctx *ctx, int64_t work)
{
  int64_t g = (work + 255) / 256;
  if (g > (int64_t)ctx->num_sms * 16) g = (int64_t)ctx->num_sms * 16;
  return (int)(g < 1 ? 1 : g);
}

#define FREE_ALL()                                            \
  do {                                                        \
    for (size_t _i = 0; _i < sizeof(bufs) / sizeof(bufs[0]); ++_i) \
      if (bufs[_i]) cudaFree(bufs[_i]);                        \
  } while (0)

extern "C" int gp_fastpca(gp_ctx *ctx, int32_t K, int32_t L, int32_t I, uint64_t seed,
                          const double *omega, const gp_xtx_opts *opts, double *evals,
                          double *evecs)
{
  if (!ctx || !opts) return GP_ERR_ARG;
  const int32_t precision = opts->precision;
  if (!ctx->d_geno || ctx->nrows < 1 || ctx->ncols < 1)
    return gp_fail(ctx, GP_ERR_STATE, "gp_fastpca: genotypes, samples and SNPs must be set first");
  if (K < 1 || L <= K || I < 1 || (int64_t)(I + 1) * L > 1024)
    return gp_fail(ctx, GP_ERR_ARG, "gp_fastpca: need 0 < K < L and 0 < I, (I+1) L <= 1024");
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  const int32_t n = ctx->nrows, nc = ctx->ncols;
  const int32_t c4 = (I + 1) * L;
  const int use_tc = precision != GP_PREC_FP64;

  /* per-SNP tables over the rows; nothing is killed but the monomorphic SNPs, whose rows of
   * X are zero anyway (setgval) */
  gp_xtx_opts o = {opts->fancynorm, opts->altnormstyle, 0, 0x7fffffff, precision};
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  int rc = gp_launch_snp_stats(ctx, &o);
  if (rc) return rc;
  std::vector<uint8_t> hk((size_t)nc);
  GP_CUDA(ctx, gp_memcpy(ctx, hk.data(), ctx->d_killed, (size_t)nc, cudaMemcpyDeviceToHost,
                         ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> kept;
  for (int32_t c = 0; c < nc; ++c)
    if (!hk[(size_t)c]) kept.push_back(c);
  const int32_t nk = (int32_t)kept.size();
  ctx->nkept = nk;
  ctx->codes4_rows = 0;
  if (nk < 1) return gp_fail(ctx, GP_ERR_NODATA, "gp_fastpca: no polymorphic SNP");
  GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_kept, kept.data(), sizeof(int32_t) * (size_t)nk,
                         cudaMemcpyHostToDevice, ctx->stream));

  /* buffers for the call */
  void *bufs[11] = {NULL};
  double *d_Q, *d_G, *d_Y1, *d_Y2, *d_B, *d_BV, *d_C, *d_w, *d_vt, *d_ev;
  int32_t *d_snprec;
  size_t nQ = (size_t)nk * c4, nG = (size_t)n * L;
  size_t nY = (size_t)nk * (size_t)(c4 > L ? c4 : L);
  cudaError_t e = cudaSuccess;
  e = cudaMalloc((void **)&d_Q, sizeof(double) * nQ); bufs[0] = d_Q;
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_G, sizeof(double) * nG * 2); bufs[1] = d_G; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_Y1, sizeof(double) * nY); bufs[2] = d_Y1; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_Y2, sizeof(double) * nY); bufs[3] = d_Y2; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_B, sizeof(double) * (size_t)n * c4); bufs[4] = d_B; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_BV, sizeof(double) * (size_t)n * c4); bufs[5] = d_BV; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_C, sizeof(double) * (size_t)c4 * c4 + 4096); bufs[6] = d_C; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_w, sizeof(double) * (size_t)c4 + 256); bufs[7] = d_w; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_vt, sizeof(double) * 4 * (size_t)nk + 256); bufs[8] = d_vt; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_snprec, sizeof(int32_t) * (size_t)nk + 256); bufs[9] = d_snprec; }
  if (e == cudaSuccess) { e = cudaMalloc((void **)&d_ev, sizeof(double) * (size_t)n * K + 256); bufs[10] = d_ev; }
  if (e != cudaSuccess) {
    FREE_ALL();
    return gp_fail(ctx, GP_ERR_NOMEM, "gp_fastpca: device allocation failed: %s", cudaGetErrorString(e));
  }
#define CK(call)                \
  do {                          \
    rc = (call);                \
    if (rc) {                   \
      FREE_ALL();               \
      return rc;                \
    }                           \
  } while (0)
#define CKC(call)                                           \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) {                                \
      FREE_ALL();                                           \
      return gp_cuda_fail(ctx, _e, #call);                  \
    }                                                       \
  } while (0)

  k_fast_vtab<<<grid_for_fast(ctx, nk), 256, 0, ctx->stream>>>(ctx->d_kept, nk, ctx->d_cols,
                                                              ctx->d_vtab, d_snprec, d_vt);
  CKC(cudaGetLastError());

  /* Omega */
  {
    std::vector<double> om((size_t)n * L);
    if (omega)
      memcpy(om.data(), omega, sizeof(double) * om.size());
    else
      make_omega(seed, n, L, om.data());
    CKC(gp_memcpy(ctx, d_G, om.data(), sizeof(double) * om.size(), cudaMemcpyHostToDevice,
                  ctx->stream));
    CKC(cudaStreamSynchronize(ctx->stream));
  }

  /* code operands: X G reads SNP rows (the device records when every sample is selected, in
   * order), X^T Q reads sample rows */
  gp_tc_codes A_snp, A_samp;
  uint8_t *codes_samp = NULL, *codes_snp = NULL;
  if (use_tc) {
    int64_t ldc;
    int32_t rows_pad;
    gp_tc_code_bytes(1, n, nk, &ldc, &rows_pad);
    CKC(cudaMalloc((void **)&codes_samp, (size_t)rows_pad * ldc + 256));
    CK(gp_tc_build_codes(ctx, 1, ctx->d_rows, n, d_snprec, nk, codes_samp, &A_samp));
    int all_rows = (n == ctx->nind_all);
    if (all_rows) {
      A_snp.codes = ctx->d_geno;
      A_snp.ldc = ctx->rlen_dev;
      A_snp.row_map = d_snprec;
      A_snp.nrows = nk;
      A_snp.k0 = n;
    } else {
      gp_tc_code_bytes(0, n, nk, &ldc, &rows_pad);
      e = cudaMalloc((void **)&codes_snp, (size_t)rows_pad * ldc + 256);
      if (e != cudaSuccess) {
        cudaFree(codes_samp);
        FREE_ALL();
        return gp_fail(ctx, GP_ERR_NOMEM, "gp_fastpca: code operand allocation failed");
      }
      rc = gp_tc_build_codes(ctx, 0, ctx->d_rows, n, d_snprec, nk, codes_snp, &A_snp);
      if (rc) {
        cudaFree(codes_samp);
        cudaFree(codes_snp);
        FREE_ALL();
        return rc;
      }
    }
  }
  int result = GP_OK;
  double *G0 = d_G, *G1 = d_G + nG;
  const int64_t ldq = nk;
  for (int32_t it = 0; it <= I && result == GP_OK; ++it) {
    /* Q_it = X G0 */
    if (use_tc) {
      gp_tc_panel pg = {G0, L, 1.0, 1};
      result = gp_geno_panel_tc_codes(ctx, &A_snp, 1, &pg, L, d_Y1, L);
      if (!result) {
        pg.count = 0;
        result = gp_geno_panel_tc_codes(ctx, &A_snp, 1, &pg, L, d_Y2, L);
      }
      if (!result) {
        k_fast_combine_xg<<<grid_for_fast(ctx, (int64_t)nk * L), 256, 0, ctx->stream>>>(
            d_Q, ldq, it * L, d_Y1, d_Y2, ctx->d_kept, ctx->d_xfancy, ctx->d_xmean, nk, L, INV_SQRT2);
      }
    } else {
      result = gp_geno_gemm_f64(ctx, 0, ctx->d_rows, n, d_snprec, d_vt, nk, G0, L, L, d_Y1, L);
      if (!result)
        k_fast_scatter<<<grid_for_fast(ctx, (int64_t)nk * L), 256, 0, ctx->stream>>>(d_Q, ldq, it * L,
                                                                                    d_Y1, nk, L);
    }
    if (result) break;
    if (it == I) break;
    /* G1 = X^T Q_it / M */
    if (use_tc) {
      k_fast_panels<<<grid_for_fast(ctx, (int64_t)nk * L), 256, 0, ctx->stream>>>(
          d_Y1, d_Y2, d_Q, ldq, it * L, L, ctx->d_kept, ctx->d_xfancy, ctx->d_xmean, nk);
      gp_tc_panel pp[2] = {{d_Y1, L, 1.0, 1}, {d_Y2, L, -1.0, 0}};
      result = gp_geno_panel_tc_codes(ctx, &A_samp, 2, pp, L, G1, L);
    } else {
      k_fast_gather<<<grid_for_fast(ctx, (int64_t)nk * L), 256, 0, ctx->stream>>>(d_Y1, d_Q, ldq,
                                                                                 it * L, L, nk);
      result = gp_geno_gemm_f64(ctx, 1, ctx->d_rows, n, d_snprec, d_vt, nk, d_Y1, L, L, G1, L);
    }
    if (result) break;
    k_scale_copy<<<grid_for_fast(ctx, nG), 256, 0, ctx->stream>>>(G0, G1, (int64_t)nG,
                                                                  1.0 / (double)nc);
  }
  if (result) {
    if (codes_samp) cudaFree(codes_samp);
    if (codes_snp) cudaFree(codes_snp);
    FREE_ALL();
    return result;
  }

  /* orthonormal basis of Q's columns: Householder QR (geqrf + orgqr), FP64 */
  {
    int lw1 = 0, lw2 = 0;
    double *tau = d_w;
    if (cusolverDnDgeqrf_bufferSize(ctx->solver, nk, c4, d_Q, (int)ldq, &lw1) !=
            CUSOLVER_STATUS_SUCCESS ||
        cusolverDnDorgqr_bufferSize(ctx->solver, nk, c4, c4, d_Q, (int)ldq, tau, &lw2) !=
            CUSOLVER_STATUS_SUCCESS)
      result = gp_fail(ctx, GP_ERR_SOLVER, "geqrf/orgqr buffer size failed");
    double *ws = NULL;
    int *info = NULL;
    if (!result) {
      int lw = lw1 > lw2 ? lw1 : lw2;
      e = cudaMalloc((void **)&ws, sizeof(double) * (size_t)lw + 256);
      if (e != cudaSuccess) result = gp_fail(ctx, GP_ERR_NOMEM, "QR workspace allocation failed");
      info = (int *)((double *)ws + lw);
      if (!result &&
          (cusolverDnDgeqrf(ctx->solver, nk, c4, d_Q, (int)ldq, tau, ws, lw, info) !=
               CUSOLVER_STATUS_SUCCESS ||
           cusolverDnDorgqr(ctx->solver, nk, c4, c4, d_Q, (int)ldq, tau, ws, lw, info) !=
               CUSOLVER_STATUS_SUCCESS))
        result = gp_fail(ctx, GP_ERR_SOLVER, "geqrf/orgqr failed");
      if (!result) {
        int hinfo = 0;
        e = gp_memcpy(ctx, &hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess || hinfo != 0) result = gp_fail(ctx, GP_ERR_SOLVER, "orgqr info %d", hinfo);
      }
      if (ws) cudaFree(ws);
    }
  }
  /* B = X^T Q  (n x c4, row-major [i][col]) */
  if (!result) {
    double *pa = NULL, *pb = NULL;
    e = cudaMalloc((void **)&pa, sizeof(double) * nQ * 2);
    if (e != cudaSuccess) result = gp_fail(ctx, GP_ERR_NOMEM, "panel allocation failed");
    if (!result) {
      pb = pa + nQ;
      if (use_tc) {
        k_fast_panels<<<grid_for_fast(ctx, (int64_t)nQ), 256, 0, ctx->stream>>>(
            pa, pb, d_Q, ldq, 0, c4, ctx->d_kept, ctx->d_xfancy, ctx->d_xmean, nk);
        gp_tc_panel pp[2] = {{pa, c4, 1.0, 1}, {pb, c4, -1.0, 0}};
        result = gp_geno_panel_tc_codes(ctx, &A_samp, 2, pp, c4, d_B, c4);
      } else {
        k_fast_gather<<<grid_for_fast(ctx, (int64_t)nQ), 256, 0, ctx->stream>>>(pa, d_Q, ldq, 0, c4,
                                                                               nk);
        result = gp_geno_gemm_f64(ctx, 1, ctx->d_rows, n, d_snprec, d_vt, nk, pa, c4, c4, d_B, c4);
      }
      cudaFree(pa);
    }
  }
  /* C = B^T B (c4 x c4), eigen-decomposition, U_K = B V_K / S_K */
  if (!result) {
    if (!ctx->blas) {
      if (cublasCreate(&ctx->blas) != CUBLAS_STATUS_SUCCESS)
        result = gp_fail(ctx, GP_ERR_SOLVER, "cublasCreate failed");
      else
        cublasSetStream(ctx->blas, ctx->stream);
    }
    const double one = 1.0, zero = 0.0;
    /* B row-major n x c4 = column-major c4 x n (Bc); C = Bc Bc^T */
    if (!result &&
        cublasDgemm(ctx->blas, CUBLAS_OP_N, CUBLAS_OP_T, c4, c4, n, &one, d_B, c4, d_B, c4, &zero,
                    d_C, c4) != CUBLAS_STATUS_SUCCESS)
      result = gp_fail(ctx, GP_ERR_SOLVER, "cublasDgemm (B^T B) failed");
    int lw = 0;
    if (!result &&
        cusolverDnDsyevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                    c4, d_C, c4, d_w, &lw) != CUSOLVER_STATUS_SUCCESS)
      result = gp_fail(ctx, GP_ERR_SOLVER, "syevd buffer size failed");
    double *ws = NULL;
    if (!result) {
      e = cudaMalloc((void **)&ws, sizeof(double) * (size_t)lw + 256);
      if (e != cudaSuccess) result = gp_fail(ctx, GP_ERR_NOMEM, "syevd workspace allocation failed");
    }
    if (!result) {
      int *info = (int *)(ws + lw);
      if (cusolverDnDsyevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, c4, d_C,
                           c4, d_w, ws, lw, info) != CUSOLVER_STATUS_SUCCESS)
        result = gp_fail(ctx, GP_ERR_SOLVER, "syevd failed");
      /* BV (column-major n x c4) = B (row-major n x c4 = col-major c4 x n)^T V */
      if (!result &&
          cublasDgemm(ctx->blas, CUBLAS_OP_T, CUBLAS_OP_N, n, c4, c4, &one, d_B, c4, d_C, c4,
                      &zero, d_BV, n) != CUBLAS_STATUS_SUCCESS)
        result = gp_fail(ctx, GP_ERR_SOLVER, "cublasDgemm (B V) failed");
    }
    if (!result) {
      k_fast_evecs<<<grid_for_fast(ctx, (int64_t)n * K), 256, 0, ctx->stream>>>(d_ev, d_BV, n, c4,
                                                                                K, d_w);
      std::vector<double> hw((size_t)c4);
      e = gp_memcpy(ctx, hw.data(), d_w, sizeof(double) * (size_t)c4, cudaMemcpyDeviceToHost,
                    ctx->stream);
      if (e == cudaSuccess && evecs)
        e = gp_memcpy(ctx, evecs, d_ev, sizeof(double) * (size_t)n * K, cudaMemcpyDeviceToHost,
                      ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) result = gp_cuda_fail(ctx, e, "gp_fastpca read-back");
      if (!result && evals)
        for (int32_t j = 0; j < K; ++j) evals[j] = hw[(size_t)(c4 - 1 - j)] / (double)nc;
    }
    if (ws) cudaFree(ws);
  }
  if (codes_samp) cudaFree(codes_samp);
  if (codes_snp) cudaFree(codes_snp);
  FREE_ALL();
  return result;
}
