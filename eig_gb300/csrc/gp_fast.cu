/*
 * fastmode: randomized block-Krylov PCA (kjg_fpca src/ksrc/kjg_fpca.c:24-102, data table of
 * setgval src/gval.c:31-87).
 *
 *   X (M SNPs x N samples), X[s][i] = ((g - mean_s) fancy_s)/sqrt(2), missing -> 0
 *   G_0 = Omega (N x L);  for i <= I:  Q_i = X G_i,  G_{i+1} = X^T Q_i / M
 *   Q = [Q_0 .. Q_I]  (M x (I+1)L)  ->  orthonormal basis U of its columns
 *   B = X^T U  (N x (I+1)L);  top K left singular vectors of B and S^2/M
 *
 * Omega comes from GSL's default generator exactly as kjg_gsl_rng_init and
 * kjg_gsl_ran_ugaussian_matrix draw it (src/ksrc/kjg_gsl.c:100-190): MT19937 seeded with the
 * parfile's seed (GSL maps seed 0 to 4357), polar Box-Muller pairs along each row from
 * uniform_pos draws (the next 32-bit output / 2^32, zero skipped), the last column of an odd L
 * holding one uniform draw.  MT19937 is the published Matsumoto-Nishimura generator with its
 * 2002 initialisation, which std::mt19937 implements.
 *
 * Products with X use the exact sliced tensor-core products (gp_geno_tc.cu) for the split
 * precisions, written as X = (G fancy - O xmean)/sqrt(2) with G the allele counts and O the
 * observed mask (the FP64 SIMT products with the value table for GP_PREC_FP64).  The code
 * operands are built once per call; with every sample selected the SNP-major device records
 * themselves are the operand of X G.
 *
 * The basis of the Krylov space is orthonormalised block by block as it is built (block
 * classical Gram-Schmidt with reorthogonalisation, BCGS2): each new block Q_i = X G_i (M x L,
 * FP64) loses its components along the earlier orthonormal blocks, then W = Q_i^T Q_i =
 * V diag(s) V^T gives Q_i := Q_i V diag(s^-1/2) over the directions whose remaining norm is
 * above 1e-10 of the block's norm before projection (the others are numerically dependent and
 * become zero columns); the projection and the in-block step run twice.  W's decomposition is
 * a one-block cyclic Jacobi (k_block_orth).  The next block is G_{i+1} = X^T Q_i / M, which
 * spans the same Krylov space as the reference's power step from G_i, and H_i = X^T Q_i is
 * kept: B = X^T U = [H_0 .. H_I] needs no further pass over the genotypes.  B^T B =
 * V_B diag(mu) V_B^T (an FP64 tall-skinny Gram and this library's own eigensolver,
 * gp_eig_sym), eval = mu/M and the top-K left singular vectors B V_B mu^-1/2.  The reference
 * takes U from an SVD of the whole Q (kjg_gsl_SVD, which loses the early blocks once the
 * later ones are 1e16 times larger) and forms B = X^T U with another pass over the
 * genotypes; both are Rayleigh-Ritz on the same space.  All of it is FP64 on the GPU; no
 * vendor solver or BLAS is called.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <random>
#include <vector>

#include "gp_geno_gemm.h"
#include "gp_geno_tc.h"
#include "gp_internal.h"

static const double INV_SQRT2 = 0.70710678118654752440;

/* gsl_rng_uniform_pos of GSL's mt19937 */
struct gsl_mt19937 {
  std::mt19937 g;
  explicit gsl_mt19937(uint64_t seed)
      : g((std::mt19937::result_type)(seed == 0 ? 4357u : (uint32_t)(seed & 0xffffffffu))) {}
  double uniform_pos()
  {
    double x;
    do {
      x = (double)(uint32_t)g() / 4294967296.0;
    } while (x == 0.0);
    return x;
  }
};

/* Omega (N x L row-major) as kjg_gsl_ran_ugaussian_matrix fills it */
static void make_omega(uint64_t seed, int32_t n, int32_t L, double *om)
{
  gsl_mt19937 r(seed);
  for (int32_t i = 0; i < n; ++i) {
    double *row = om + (size_t)i * L;
    int32_t j = 0;
    for (; j + 1 < L; j += 2) {
      double x, y, r2;
      do {
        x = -1.0 + 2.0 * r.uniform_pos();
        y = -1.0 + 2.0 * r.uniform_pos();
        r2 = x * x + y * y;
      } while (r2 > 1.0 || r2 == 0.0);
      r2 = sqrt(-2.0 * log(r2) / r2);
      row[j] = x * r2;
      row[j + 1] = y * r2;
    }
    if (L % 2) row[j] = r.uniform_pos();
  }
}

/* Q[s][j] (row-major, L) = (fancy_s Yg[s][j] - xmean_s Yo[s][j]) / sqrt2 */
__global__ void k_fast_combine_xg(double *Q, const double *yg, const double *yo,
                                  const int32_t *kept, const double *xfancy, const double *xmean,
                                  int32_t nk, int32_t L, double scale)
{
  int64_t total = (int64_t)nk * L;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = kept[idx / L];
    Q[idx] = (xfancy[c] * yg[idx] - xmean[c] * yo[idx]) * scale;
  }
}

/* panels for X^T Q: a[s][j] = fancy_s Q[s][j] / sqrt2, b[s][j] = xmean_s Q[s][j] / sqrt2 */
__global__ void k_fast_panels(double *a, double *b, const double *Q, const int32_t *kept,
                              const double *xfancy, const double *xmean, int32_t nk, int32_t L)
{
  int64_t total = (int64_t)nk * L;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = kept[idx / L];
    double q = Q[idx] * INV_SQRT2;
    a[idx] = xfancy[c] * q;
    b[idx] = xmean[c] * q;
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

#define TSG_T 32     /* cross-product tile edge */
#define TSG_R 64     /* rows staged per step */

/*
 * Partial cross products of two tall-skinny row-major matrices A (n x ca, row stride lda) and
 * B (n x cb, row stride ldb): CTA (p, q) computes the 32 x 32 tile p of A^T B over the rows of
 * chunk q and writes it to part[q][i][j] (ca x cb); k_ts_reduce sums the chunks in order
 * (deterministic).
 */
__global__ void __launch_bounds__(256)
k_ts_cross(const double *__restrict__ A, int64_t lda, int32_t ca, const double *__restrict__ B,
           int64_t ldb, int32_t cb, int64_t n, int64_t chunk, double *part)
{
  __shared__ double As[TSG_R][TSG_T + 1];
  __shared__ double Bs[TSG_R][TSG_T + 1];
  const int32_t tb = (cb + TSG_T - 1) / TSG_T;
  const int32_t ti = (int32_t)blockIdx.x / tb, tj = (int32_t)blockIdx.x - ti * tb;
  const int32_t c0 = ti * TSG_T, d0 = tj * TSG_T;
  const int64_t r0 = (int64_t)blockIdx.y * chunk;
  const int64_t r1 = r0 + chunk < n ? r0 + chunk : n;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int64_t rs = r0; rs < r1; rs += TSG_R) {
    for (int e = tid; e < TSG_R * TSG_T; e += 256) {
      const int rr = e / TSG_T, cc = e - rr * TSG_T;
      const int64_t r = rs + rr;
      double va = 0.0, vb = 0.0;
      if (r < r1) {
        if (c0 + cc < ca) va = A[r * lda + c0 + cc];
        if (d0 + cc < cb) vb = B[r * ldb + d0 + cc];
      }
      As[rr][cc] = va;
      Bs[rr][cc] = vb;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < TSG_R; ++k) {
      const double a0 = As[k][ty], a1 = As[k][ty + 16];
      const double b0 = Bs[k][tx], b1 = Bs[k][tx + 16];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  double *o = part + (int64_t)blockIdx.y * ca * cb;
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int32_t i = c0 + ty + 16 * u, j = d0 + tx + 16 * v;
      if (i < ca && j < cb) o[(int64_t)i * cb + j] = acc[u][v];
    }
}

/* out[i][j] = sum over the chunks, in order, of part[q][i][j] (count = ca * cb) */
__global__ void k_ts_reduce(double *out, const double *part, int32_t nchunk, int64_t count)
{
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < count;
       idx += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int32_t q = 0; q < nchunk; ++q) acc += part[(int64_t)q * count + idx];
    out[idx] = acc;
  }
}

/* Q -= Qp C: Q (n x L, row stride L), Qp (n x ca, row stride ldp), C (ca x L) */
__global__ void k_ts_project(double *Q, const double *__restrict__ Qp, int64_t ldp, int32_t ca,
                             const double *__restrict__ C, int64_t n, int32_t L)
{
  const int64_t total = n * L;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / L;
    const int32_t j = (int32_t)(idx - r * L);
    double q = 0.0;
    for (int32_t k = 0; k < ca; ++k) q = fma(Qp[r * ldp + k], C[(int64_t)k * L + j], q);
    Q[idx] -= q;
  }
}

#define JAC_MAX 64 /* largest block width of the Jacobi kernel */

/*
 * One block: the L x L matrix W (symmetrised) is diagonalised by cyclic Jacobi rotations
 * (Golub & Van Loan, Matrix Computations, 8.5: the symmetric Schur decomposition of each
 * 2 x 2 pivot), W = V diag(s) V^T, and T = V diag(s^-1/2) is written for the directions with
 * s > tol * max(pre[j][j]) (max(W[j][j]) when pre is NULL; zero columns for the others).  A
 * pivot is rotated while |W_pq| > 1e-15 sqrt(|W_pp W_qq|), the threshold that keeps the small
 * eigenvalues of a positive semidefinite W to high relative accuracy (Demmel & Veselic, 1992);
 * the sweeps stop after one without a rotation, at most 40.
 */
__global__ void __launch_bounds__(JAC_MAX)
k_block_orth(const double *__restrict__ Wg, const double *__restrict__ pre, int32_t L,
             double tol, double *T)
{
  __shared__ double W[JAC_MAX][JAC_MAX + 1];
  __shared__ double V[JAC_MAX][JAC_MAX + 1];
  __shared__ double cs[2];
  __shared__ int nrot;
  const int t = threadIdx.x;
  for (int i = 0; i < L; ++i)
    if (t < L) {
      W[i][t] = 0.5 * (Wg[(int64_t)i * L + t] + Wg[(int64_t)t * L + i]);
      V[i][t] = i == t ? 1.0 : 0.0;
    }
  __syncthreads();
  for (int sweep = 0; sweep < 40; ++sweep) {
    if (t == 0) nrot = 0;
    __syncthreads();
    for (int p = 0; p < L - 1; ++p)
      for (int q = p + 1; q < L; ++q) {
        if (t == 0) {
          const double apq = W[p][q];
          double c = 1.0, sn = 0.0;
          if (apq != 0.0 && fabs(apq) > 1e-15 * sqrt(fabs(W[p][p] * W[q][q]))) {
            const double tau = (W[q][q] - W[p][p]) / (2.0 * apq);
            const double tt = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + tt * tt);
            sn = tt * c;
            ++nrot;
          }
          cs[0] = c;
          cs[1] = sn;
        }
        __syncthreads();
        const double c = cs[0], sn = cs[1];
        if (sn != 0.0) {
          if (t < L) { /* rows p, q: W := J^T W */
            const double wp = W[p][t], wq = W[q][t];
            W[p][t] = c * wp - sn * wq;
            W[q][t] = sn * wp + c * wq;
          }
          __syncthreads();
          if (t < L) { /* columns p, q: W := W J, V := V J */
            const double wp = W[t][p], wq = W[t][q];
            W[t][p] = c * wp - sn * wq;
            W[t][q] = sn * wp + c * wq;
            const double vp = V[t][p], vq = V[t][q];
            V[t][p] = c * vp - sn * vq;
            V[t][q] = sn * vp + c * vq;
          }
        }
        __syncthreads();
      }
    const bool done = nrot == 0;
    __syncthreads();
    if (done) break;
  }
  double pmax = 0.0;
  for (int i = 0; i < L; ++i)
    pmax = fmax(pmax, pre ? pre[(int64_t)i * L + i] : Wg[(int64_t)i * L + i]);
  if (t < L) {
    const double sk = W[t][t];
    const bool keep = sk > tol * pmax && sk > 0.0;
    const double f = keep ? 1.0 / sqrt(sk) : 0.0;
    for (int i = 0; i < L; ++i) T[(int64_t)i * L + t] = V[i][t] * f;
  }
}

/* out (n x L) = Q T; with qp != NULL also qp[:, col0 ..] (row stride ldp) = Q T */
__global__ void k_block_apply(const double *__restrict__ Q, const double *__restrict__ T,
                              double *out, double *qp, int64_t ldp, int32_t col0, int64_t n,
                              int32_t L)
{
  const int64_t total = n * L;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / L;
    const int32_t j = (int32_t)(idx - r * L);
    double q = 0.0;
    for (int32_t k = 0; k < L; ++k) q = fma(Q[r * L + k], T[(int64_t)k * L + j], q);
    out[idx] = q;
    if (qp) qp[r * ldp + col0 + j] = q;
  }
}

/* G := Hp[:, col0 ..] / M (the next block) */
__global__ void k_block_next(double *G, const double *__restrict__ Hp, int64_t ldp, int32_t col0,
                             int64_t n, int32_t L, double inv_m)
{
  const int64_t total = n * L;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / L;
    const int32_t j = (int32_t)(idx - r * L);
    G[idx] = Hp[r * ldp + col0 + j] * inv_m;
  }
}

/* C := (C + C^T) / 2 (n x n) */
__global__ void k_symmetrize(double *C, int32_t n)
{
  const int64_t total = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = (int32_t)(idx / n), j = (int32_t)(idx - (int64_t)i * n);
    if (i < j) {
      const double v = 0.5 * (C[idx] + C[(int64_t)j * n + i]);
      C[idx] = v;
      C[(int64_t)j * n + i] = v;
    }
  }
}

/* evec[j][i] = sum_c Hp[i][c] U[j][c] / sqrt(mu_j) */
__global__ void k_fast_evecs(double *evecs, const double *__restrict__ Hp, int64_t ldp,
                             const double *__restrict__ U, const double *__restrict__ mu,
                             int64_t n, int32_t c4, int32_t K)
{
  const int64_t total = n * K;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t j = (int32_t)(idx / n);
    const int64_t i = idx - (int64_t)j * n;
    double acc = 0.0;
    for (int32_t c = 0; c < c4; ++c) acc = fma(Hp[i * ldp + c], U[(int64_t)j * c4 + c], acc);
    evecs[idx] = mu[j] > 0.0 ? acc / sqrt(mu[j]) : 0.0;
  }
}

static int grid_for_fast(const gp_ctx *ctx, int64_t work)
{
  int64_t g = (work + 255) / 256;
  if (g > (int64_t)ctx->num_sms * 16) g = (int64_t)ctx->num_sms * 16;
  return (int)(g < 1 ? 1 : g);
}

/* out (ca x cb) = A^T B over n rows, through the chunk partials in part (deterministic) */
static int ts_cross(gp_ctx *ctx, const double *A, int64_t lda, int32_t ca, const double *B,
                    int64_t ldb, int32_t cb, int64_t n, double *part, size_t part_cap,
                    double *out)
{
  const int32_t ntiles = ((ca + TSG_T - 1) / TSG_T) * ((cb + TSG_T - 1) / TSG_T);
  int64_t want = ((int64_t)ctx->num_sms * 4 + ntiles - 1) / ntiles;
  int64_t chunk = (n + want - 1) / want;
  if (chunk < 2048) chunk = 2048;
  int64_t nchunk = (n + chunk - 1) / chunk;
  while ((size_t)(nchunk * ca * cb) > part_cap) { /* fewer, longer chunks when space is short */
    chunk *= 2;
    nchunk = (n + chunk - 1) / chunk;
  }
  dim3 grid((unsigned)ntiles, (unsigned)nchunk);
  k_ts_cross<<<grid, 256, 0, ctx->stream>>>(A, lda, ca, B, ldb, cb, n, chunk, part);
  GP_LAUNCH_CHECK(ctx, "k_ts_cross");
  k_ts_reduce<<<grid_for_fast(ctx, (int64_t)ca * cb), 256, 0, ctx->stream>>>(out, part,
                                                                             (int32_t)nchunk,
                                                                             (int64_t)ca * cb);
  GP_LAUNCH_CHECK(ctx, "k_ts_reduce");
  return GP_OK;
}

/* a direction of a new Krylov block is dependent on the earlier blocks when its norm after
 * projection is below 1e-10 of the block's norm before it (s is a squared norm) */
#define GP_FAST_DEP_TOL 1e-20

/* device buffers of one gp_fastpca call, freed together */
struct fast_bufs {
  std::vector<void *> p;
  ~fast_bufs()
  {
    for (void *q : p)
      if (q) cudaFree(q);
  }
  template <class T> cudaError_t get(T **out, size_t count)
  {
    void *q = NULL;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 256);
    p.push_back(q);
    *out = (T *)q;
    return e;
  }
};

extern "C" int gp_fastpca(gp_ctx *ctx, int32_t K, int32_t L, int32_t I, uint64_t seed,
                          const double *omega, const gp_xtx_opts *opts, double *evals,
                          double *evecs)
{
  if (!ctx || !opts) return GP_ERR_ARG;
  const int32_t precision = opts->precision;
  if (!ctx->d_geno || ctx->nrows < 1 || ctx->ncols < 1)
    return gp_fail(ctx, GP_ERR_STATE, "gp_fastpca: genotypes, samples and SNPs must be set first");
  if (K < 1 || L <= K || L > JAC_MAX || I < 1 || (int64_t)(I + 1) * L > 1024)
    return gp_fail(ctx, GP_ERR_ARG,
                   "gp_fastpca: need 0 < K < L <= 64 and 0 < I, (I+1) L <= 1024");
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

  /* buffers: the orthonormal blocks Q_i (nk x c4) and H_i = X^T Q_i (n x c4) side by side,
   * the next G (n x L), the current block and two product panels (nk x L), cross-product
   * partials and the small matrices */
  const size_t nG = (size_t)n * L, nQ = (size_t)nk * L;
  const int64_t nmax = n > nk ? n : nk;
  /* chunk partials: ts_cross takes chunks of at least 2,048 rows and about four CTAs per SM
   * (it lengthens the chunks when this is short) */
  const size_t part_cap = (size_t)c4 * c4 + ((size_t)nmax / 2048 + 2) * (size_t)c4 * L +
                          (size_t)4 * ctx->num_sms * TSG_T * TSG_T + 4096;
  fast_bufs B;
  double *d_Qp, *d_Hp, *d_G, *d_Q, *d_Y1, *d_Y2, *d_part, *d_C, *d_W, *d_pre, *d_T, *d_mu,
      *d_U, *d_ev, *d_vt;
  int32_t *d_snprec;
  cudaError_t e = B.get(&d_Qp, (size_t)nk * c4);
  if (e == cudaSuccess) e = B.get(&d_Hp, (size_t)n * c4);
  if (e == cudaSuccess) e = B.get(&d_G, nG);
  if (e == cudaSuccess) e = B.get(&d_Q, nQ);
  if (e == cudaSuccess) e = B.get(&d_Y1, nQ);
  if (e == cudaSuccess) e = B.get(&d_Y2, nQ);
  if (e == cudaSuccess) e = B.get(&d_part, part_cap);
  if (e == cudaSuccess) e = B.get(&d_C, (size_t)c4 * c4);
  if (e == cudaSuccess) e = B.get(&d_W, (size_t)L * L);
  if (e == cudaSuccess) e = B.get(&d_pre, (size_t)L * L);
  if (e == cudaSuccess) e = B.get(&d_T, (size_t)L * L);
  if (e == cudaSuccess) e = B.get(&d_mu, (size_t)c4);
  if (e == cudaSuccess) e = B.get(&d_U, (size_t)K * c4);
  if (e == cudaSuccess) e = B.get(&d_ev, (size_t)n * K);
  if (e == cudaSuccess) e = B.get(&d_vt, 4 * (size_t)nk);
  if (e == cudaSuccess) e = B.get(&d_snprec, (size_t)nk);
  if (e != cudaSuccess)
    return gp_fail(ctx, GP_ERR_NOMEM, "gp_fastpca: device allocation failed: %s",
                   cudaGetErrorString(e));

  k_fast_vtab<<<grid_for_fast(ctx, nk), 256, 0, ctx->stream>>>(ctx->d_kept, nk, ctx->d_cols,
                                                              ctx->d_vtab, d_snprec, d_vt);
  GP_LAUNCH_CHECK(ctx, "k_fast_vtab");

  /* Omega = G_0 */
  {
    std::vector<double> om(nG);
    if (omega)
      memcpy(om.data(), omega, sizeof(double) * om.size());
    else
      make_omega(seed, n, L, om.data());
    GP_CUDA(ctx, gp_memcpy(ctx, d_G, om.data(), sizeof(double) * om.size(),
                           cudaMemcpyHostToDevice, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }

  /* code operands: X G reads SNP rows (the device records when every sample is selected, in
   * order), X^T Q reads sample rows */
  gp_tc_codes A_snp, A_samp;
  uint8_t *codes_samp = NULL, *codes_snp = NULL;
  if (use_tc) {
    int64_t ldc;
    int32_t rows_pad;
    gp_tc_code_bytes(1, n, nk, &ldc, &rows_pad);
    GP_CUDA(ctx, B.get(&codes_samp, (size_t)rows_pad * ldc));
    rc = gp_tc_build_codes(ctx, 1, ctx->d_rows, n, d_snprec, nk, codes_samp, &A_samp);
    if (rc) return rc;
    if (n == ctx->nind_all) {
      A_snp.codes = ctx->d_geno;
      A_snp.ldc = ctx->rlen_dev;
      A_snp.row_map = d_snprec;
      A_snp.nrows = nk;
      A_snp.k0 = n;
    } else {
      gp_tc_code_bytes(0, n, nk, &ldc, &rows_pad);
      e = B.get(&codes_snp, (size_t)rows_pad * ldc);
      if (e != cudaSuccess)
        return gp_fail(ctx, GP_ERR_NOMEM, "gp_fastpca: code operand allocation failed");
      rc = gp_tc_build_codes(ctx, 0, ctx->d_rows, n, d_snprec, nk, codes_snp, &A_snp);
      if (rc) return rc;
    }
  }
  /* the Krylov blocks, orthonormalised as they come: Q_i = X G_i, H_i = X^T Q_i */
  for (int32_t it = 0; it <= I; ++it) {
    if (use_tc) {
      gp_tc_panel pg = {d_G, L, 1.0, 1};
      rc = gp_geno_panel_tc_codes(ctx, &A_snp, 1, &pg, L, d_Y1, L);
      if (rc) return rc;
      pg.count = 0;
      rc = gp_geno_panel_tc_codes(ctx, &A_snp, 1, &pg, L, d_Y2, L);
      if (rc) return rc;
      k_fast_combine_xg<<<grid_for_fast(ctx, (int64_t)nQ), 256, 0, ctx->stream>>>(
          d_Q, d_Y1, d_Y2, ctx->d_kept, ctx->d_xfancy, ctx->d_xmean, nk, L, INV_SQRT2);
      GP_LAUNCH_CHECK(ctx, "k_fast_combine_xg");
    } else {
      rc = gp_geno_gemm_f64(ctx, 0, ctx->d_rows, n, d_snprec, d_vt, nk, d_G, L, L, d_Q, L);
      if (rc) return rc;
    }
    /* BCGS2: (project against the earlier blocks, orthonormalise within the block) twice;
     * the first pass drops directions below 1e-10 of the block's norm before projection */
    const int32_t ca = it * L;
    rc = ts_cross(ctx, d_Q, L, L, d_Q, L, L, nk, d_part, part_cap, d_pre);
    if (rc) return rc;
    for (int pass = 0; pass < 2; ++pass) {
      if (ca > 0) {
        rc = ts_cross(ctx, d_Qp, c4, ca, d_Q, L, L, nk, d_part, part_cap, d_C);
        if (rc) return rc;
        k_ts_project<<<grid_for_fast(ctx, (int64_t)nQ), 256, 0, ctx->stream>>>(
            d_Q, d_Qp, c4, ca, d_C, nk, L);
        GP_LAUNCH_CHECK(ctx, "k_ts_project");
      }
      rc = ts_cross(ctx, d_Q, L, L, d_Q, L, L, nk, d_part, part_cap, d_W);
      if (rc) return rc;
      k_block_orth<<<1, JAC_MAX, 0, ctx->stream>>>(d_W, pass == 0 ? d_pre : NULL, L,
                                                  GP_FAST_DEP_TOL, d_T);
      GP_LAUNCH_CHECK(ctx, "k_block_orth");
      k_block_apply<<<grid_for_fast(ctx, (int64_t)nQ), 256, 0, ctx->stream>>>(
          d_Q, d_T, d_Y1, pass == 1 ? d_Qp : NULL, c4, ca, nk, L);
      GP_LAUNCH_CHECK(ctx, "k_block_apply");
      double *tq = d_Q;
      d_Q = d_Y1;
      d_Y1 = tq;
    }
    /* H_i = X^T Q_i into its columns of Hp; the next block G = H_i / M */
    if (use_tc) {
      k_fast_panels<<<grid_for_fast(ctx, (int64_t)nQ), 256, 0, ctx->stream>>>(
          d_Y1, d_Y2, d_Q, ctx->d_kept, ctx->d_xfancy, ctx->d_xmean, nk, L);
      GP_LAUNCH_CHECK(ctx, "k_fast_panels");
      gp_tc_panel pp[2] = {{d_Y1, L, 1.0, 1}, {d_Y2, L, -1.0, 0}};
      rc = gp_geno_panel_tc_codes(ctx, &A_samp, 2, pp, L, d_Hp + ca, c4);
      if (rc) return rc;
    } else {
      rc = gp_geno_gemm_f64(ctx, 1, ctx->d_rows, n, d_snprec, d_vt, nk, d_Q, L, L, d_Hp + ca,
                            c4);
      if (rc) return rc;
    }
    if (it < I) {
      k_block_next<<<grid_for_fast(ctx, (int64_t)nG), 256, 0, ctx->stream>>>(
          d_G, d_Hp, c4, ca, n, L, 1.0 / (double)nc);
      GP_LAUNCH_CHECK(ctx, "k_block_next");
    }
  }
  /* B = X^T U = Hp; B^T B = V diag(mu) V^T; eval = mu / M, evec = B v / sqrt(mu) */
  rc = ts_cross(ctx, d_Hp, c4, c4, d_Hp, c4, c4, n, d_part, part_cap, d_C);
  if (rc) return rc;
  k_symmetrize<<<grid_for_fast(ctx, (int64_t)c4 * c4), 256, 0, ctx->stream>>>(d_C, c4);
  GP_LAUNCH_CHECK(ctx, "k_symmetrize");
  rc = gp_eig_sym(ctx, d_C, c4, K, d_mu, d_U);
  if (rc) return rc;
  k_fast_evecs<<<grid_for_fast(ctx, (int64_t)n * K), 256, 0, ctx->stream>>>(d_ev, d_Hp, c4, d_U,
                                                                           d_mu, n, c4, K);
  GP_LAUNCH_CHECK(ctx, "k_fast_evecs");
  std::vector<double> hmu((size_t)K);
  GP_CUDA(ctx, gp_memcpy(ctx, hmu.data(), d_mu, sizeof(double) * (size_t)K,
                         cudaMemcpyDeviceToHost, ctx->stream));
  if (evecs)
    GP_CUDA(ctx, gp_memcpy(ctx, evecs, d_ev, sizeof(double) * (size_t)n * K,
                           cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (evals)
    for (int32_t j = 0; j < K; ++j) evals[j] = hmu[(size_t)j] / (double)nc;
  return GP_OK;
}
