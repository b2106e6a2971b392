/*
 * Dense symmetric FP64 eigensolve for the smartpca Gram, on the device: all N eigenvalues
 * and the top nvec eigenvectors (the reference computes every eigenpair with LAPACK dspev,
 * src/eigensrc/eigx.c:97-117, but prints all eigenvalues and uses only the top vectors).
 *
 *   1. Householder tridiagonalisation A = Q T Q^T (cuSOLVER sytrd, lower);
 *   2. all eigenvalues of T by multisection on Sturm counts (the published bisection method:
 *      the count of negative pivots of the LDL^T factorisation of T - x I equals the number
 *      of eigenvalues below x), several lanes per eigenvalue index: FP32 brackets first,
 *      checked and finished in FP64 to 1e-13 ||T||;
 *   3. the top nvec eigenvectors of T by inverse iteration, one block per vector: LU with
 *      partial pivoting of the tridiagonal T - lambda I (Gaussian elimination with row
 *      interchanges) and three solves from a fixed pseudo-random start, then modified
 *      Gram-Schmidt over the vectors in order (eigenvalues that are distinct to far more than
 *      eps*||T|| make each iterate converge to its own eigenvector);
 *   4. back-transformation of those nvec vectors only, V = Q Z (cuSOLVER ormtr).
 */
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "gp_internal.h"
#include "gp_tc.cuh"


/* the same count in FP32 (coarse brackets only; verified in FP64 afterwards) */
__device__ __forceinline__ int sturm_count_f(const float *d, const float *e2, int n, float x,
                                             float pivmin)
{
  int cnt = 0;
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  if (q < 0.f) ++cnt;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - __fdividef(e2[i - 1], q);
    if (fabsf(q) < pivmin) q = -pivmin;
    if (q < 0.f) ++cnt;
  }
  return cnt;
}

/*
 * 1/q to ~2^-44 relative with four integer-built pieces and two FP64 FMAs: the mantissa of q
 * (truncated to 23 bits) is inverted by the FP32 approximate reciprocal, the exponent is
 * negated in integer arithmetic, and one Newton step r = r0 + r0 (1 - q r0) refines it.
 * Valid for normal q with |exponent| < 1000 (the Sturm pivots are clamped away from 0).
 * GB300's FP64 pipe is narrow, so this keeps conversions and divisions off it.
 */
__device__ __forceinline__ double rcp_newton(double q)
{
  const unsigned long long qb = (unsigned long long)__double_as_longlong(q);
  const unsigned hi = (unsigned)(qb >> 32);
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023;
  const float f = __uint_as_float(0x3F800000u | (unsigned)((qb >> 29) & 0x7FFFFFull));
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(f));
  const unsigned rb = __float_as_uint(rf);
  const unsigned er = (unsigned)((int)(rb >> 23) - 127 - e + 1023);
  const unsigned long long r0b =
      ((unsigned long long)((hi & 0x80000000u) | (er << 20) | ((rb & 0x7FFFFFu) >> 3)) << 32) |
      ((unsigned long long)(rb & 7u) << 29);
  const double r0 = __longlong_as_double((long long)r0b);
  return fma(r0, fma(-q, r0, 1.0), r0);
}

/*
 * Sturm count with 4 FP64-pipe operations per step (d - x and three FMAs); the pivot clamp
 * and the sign test work on the bit patterns.
 */
__device__ __forceinline__ int sturm_count_bits(const double *d, const double *e2, int n, double x,
                                                double pivmin)
{
  const unsigned long long piv_bits = (unsigned long long)__double_as_longlong(pivmin);
  const double negpiv = -pivmin;
  int cnt = 0;
  double q = d[0] - x;
  unsigned long long qb = (unsigned long long)__double_as_longlong(q);
  if ((qb & 0x7FFFFFFFFFFFFFFFull) < piv_bits) {
    q = negpiv;
    qb = (unsigned long long)__double_as_longlong(negpiv);
  }
  cnt += (int)(qb >> 63);
  for (int i = 1; i < n; ++i) {
    const double r = rcp_newton(q);
    q = fma(-e2[i - 1], r, d[i] - x);
    qb = (unsigned long long)__double_as_longlong(q);
    if ((qb & 0x7FFFFFFFFFFFFFFFull) < piv_bits) {
      q = negpiv;
      qb = (unsigned long long)__double_as_longlong(negpiv);
    }
    cnt += (int)(qb >> 63);
  }
  return cnt;
}

/*
 * All eigenvalues by multisection: a warp owns epw consecutive eigenvalue indices and each
 * index gets P = 32/epw lanes (P >= 1), so every warp slot of the GPU has work whatever N is.
 * A step evaluates P interior points of the bracket at once (one Sturm count per lane) and
 * keeps the sub-interval where the count crosses k: log2(P+1) bits per step.  FP32 counts
 * narrow the bracket to ~4e-7 ||T||, it is widened by 64 eps_32 ||T|| and checked with two
 * FP64 counts (back to the Gershgorin bracket if the check fails), then FP64 counts narrow it
 * to tol.  Grid: one CTA of 4 warps per SM; d, e2 and FP32 copies in shared memory
 * (24 N bytes) when they fit.
 */
__global__ void __launch_bounds__(128)
k_multisect(const double *gd, const double *ge2, int n, double gl, double gu, double tnorm,
            double pivmin, double tol, int use_smem, int epw, int P, double *w)
{
  extern __shared__ double sm[];
  const double *d = gd, *e2 = ge2;
  const float *df = NULL, *e2f = NULL;
  if (use_smem) {
    double *sd = sm, *se2 = sm + n;
    float *sdf = (float *)(sm + 2 * n), *se2f = sdf + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      sd[i] = gd[i];
      sdf[i] = (float)gd[i];
      if (i < n - 1) {
        se2[i] = ge2[i];
        se2f[i] = (float)ge2[i];
      }
    }
    __syncthreads();
    d = sd;
    e2 = se2;
    df = sdf;
    e2f = se2f;
  }
  const int lane = threadIdx.x & 31;
  const int gwarp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int slot = lane / P, sub = lane - slot * P;
  if (slot >= epw) return;
  const int k = gwarp * epw + slot;
  if (k >= n) return;
  const unsigned gmask = ((P == 32) ? 0xFFFFFFFFu : ((1u << P) - 1u)) << (slot * P);
  const int gshift = slot * P;
  const unsigned gbits = (P == 32) ? 0xFFFFFFFFu : ((1u << P) - 1u);
  double lo = gl, hi = gu;
  if (df) {
    float flo = (float)gl, fhi = (float)gu;
    const float fpiv = fmaxf((float)pivmin, 1e-30f) * 1e6f;
    const float ftol = 4e-7f * (float)tnorm;
    for (int it = 0; it < 64 && fhi - flo > ftol; ++it) {
      const float wdt = fhi - flo;
      const float x = flo + wdt * (float)(sub + 1) / (float)(P + 1);
      const int flag = (x > flo && x < fhi) ? (sturm_count_f(df, e2f, n, x, fpiv) > k) : (x >= fhi);
      const unsigned b = (__ballot_sync(gmask, flag) >> gshift) & gbits;
      const int first = b ? __ffs(b) - 1 : P;
      const float nlo = first == 0 ? flo : flo + wdt * (float)first / (float)(P + 1);
      const float nhi = first == P ? fhi : flo + wdt * (float)(first + 1) / (float)(P + 1);
      if (!(nhi - nlo < wdt)) break;
      flo = nlo;
      fhi = nhi;
    }
    const double margin = 64.0 * (double)FLT_EPSILON * tnorm;
    lo = fmax(gl, (double)flo - margin);
    hi = fmin(gu, (double)fhi + margin);
    int ok = 1;
    if (sub < 2) {
      const double x = sub == 0 ? lo : hi;
      const int c = sturm_count_bits(d, e2, n, x, pivmin);
      ok = sub == 0 ? (c <= k) : (c > k);
    }
    const unsigned bad = (__ballot_sync(gmask, !ok) >> gshift) & gbits;
    if (bad) {
      lo = gl;
      hi = gu;
    }
  }
  for (int it = 0; it < 200 && hi - lo > tol; ++it) {
    const double wdt = hi - lo;
    const double x = lo + wdt * (double)(sub + 1) / (double)(P + 1);
    const int flag = (x > lo && x < hi) ? (sturm_count_bits(d, e2, n, x, pivmin) > k) : (x >= hi);
    const unsigned b = (__ballot_sync(gmask, flag) >> gshift) & gbits;
    const int first = b ? __ffs(b) - 1 : P;
    const double nlo = first == 0 ? lo : lo + wdt * (double)first / (double)(P + 1);
    const double nhi = first == P ? hi : lo + wdt * (double)(first + 1) / (double)(P + 1);
    if (!(nhi - nlo < wdt)) break;
    lo = nlo;
    hi = nhi;
  }
  if (sub == 0) w[k] = 0.5 * (lo + hi);
}

/* ---------------------------------------------------------------------------------- */
/*
 * Householder tridiagonalisation A = Q T Q^T of the symmetric n x n matrix (lower triangle,
 * column-major: element (r, q), r >= q, at A[q*n + r]), the unblocked algorithm of LAPACK
 * dsytd2 (lower) restated for one cooperative launch:
 *   for c = 0 .. n-2:  x = A(c+1:n, c);  (beta, tau, v) = reflector of x (dlarfg: v(c+1) = 1,
 *   beta = -sign(alpha) ||x||, tau = (beta - alpha)/beta, v = x/(alpha - beta) below);
 *   y = A(c+1:n, c+1:n) v;  w = tau y - (tau^2/2)(y.v) v;  A(c+1:n, c+1:n) -= v w^T + w v^T.
 * The rank-2 update of step c is not a pass of its own: it is applied while step c+1 reads the
 * trailing matrix for its product (look-ahead), so each step reads and writes the lower
 * triangle once and reads it once more.  Per step, with the blocks' row/column ranges
 * balanced by element count:
 *   A   column c gets the pending update; w of step c-1; v of step c-1 stored into A(:, c-1)
 *       (LAPACK's reflector storage, e(c-1) on the subdiagonal); partial ||x||^2
 *   --- grid barrier
 *   B1  each block, per owned column r of the trailing matrix: pending update of A(r:n, r),
 *       written back, and y(r) = A(r:n, r) . v (lower part incl. diagonal), warp per column
 *   --- grid barrier
 *   B2  each block, per owned row r: y(r) += A(r, c+1:r) . v (strictly lower part; lanes
 *       over rows, so the loads stay coalesced in column-major), partial y.v
 *   --- grid barrier
 * Every sum has a fixed order (no atomics), so the result is deterministic.  The grid
 * barriers are counter + generation words with a %globaltimer bound: on expiry the kernel
 * records an error code and returns (the host reports GP_ERR_TIMEOUT).
 * Outputs: d[n], e[n-1], tau[n-1] and the reflectors in A, as cusolverDnDormtr(lower) reads
 * them.  Shared memory: v(step c-1), w(step c-1), v(step c) over the rows (24 n bytes).
 */
#define TR_THREADS 256
#define TR_WARPS (TR_THREADS / 32)
#define TR_ERR_BARRIER 11

__device__ __forceinline__ bool tr_grid_sync(unsigned *count, unsigned *gen, int *err)
{
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned *vgen = gen;
    volatile int *verr = err;
    const unsigned g = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      const uint64_t t0 = globaltimer_ns();
      while (*vgen == g) {
        if (*verr) {
          ok = 0;
          break;
        }
        if (globaltimer_ns() - t0 > GP_WAIT_NS) {
          atomicExch(err, TR_ERR_BARRIER);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    if (*verr) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

/* sum of the G block partials in a fixed order (warp 0), broadcast through shared memory */
__device__ __forceinline__ double tr_sum_partials(const double *part, int G, double *slot)
{
  if (threadIdx.x < 32) {
    double s = 0.0;
    for (int g = threadIdx.x; g < G; g += 32) s += part[g];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if (threadIdx.x == 0) *slot = s;
  }
  __syncthreads();
  const double r = *slot;
  __syncthreads();
  return r;
}

/* block sum of one value per thread (fixed order), result valid in thread 0 */
__device__ __forceinline__ double tr_block_sum(double v, double *red)
{
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < TR_WARPS; ++w) s += red[w];
  __syncthreads();
  return s;
}

/* start of block b's share of [0, m) when column u weighs (m - u) (B1) */
__device__ __forceinline__ int tr_split_cols(int m, int b, int G)
{
  if (b <= 0) return 0;
  if (b >= G) return m;
  const double tot = 0.5 * (double)m * (double)(m + 1);
  const double t = tot * (double)b / (double)G;
  const double a = 2.0 * (double)m + 1.0;
  double u = 0.5 * (a - sqrt(fmax(a * a - 8.0 * t, 0.0)));
  int iu = (int)ceil(u - 1e-9);
  return iu < 0 ? 0 : (iu > m ? m : iu);
}

/* start of block b's share of [0, m) when row u weighs u (B2) */
__device__ __forceinline__ int tr_split_rows(int m, int b, int G)
{
  if (b <= 0) return 0;
  if (b >= G) return m;
  const double tot = 0.5 * (double)m * (double)(m - 1);
  const double t = tot * (double)b / (double)G;
  double u = 0.5 * (1.0 + sqrt(1.0 + 8.0 * t));
  int iu = (int)ceil(u - 1e-9);
  return iu < 0 ? 0 : (iu > m ? m : iu);
}

__global__ void __launch_bounds__(TR_THREADS, 1)
k_tridiag(double *A, int n, double *d, double *e, double *tau, double *wbuf, double *ybuf,
          double *part_norm, double *part_dot, unsigned *bar, int *err)
{
  extern __shared__ double sh[];
  double *svp = sh, *swp = sh + n, *svc = sh + 2 * n;
  __shared__ double red[TR_WARPS];
  __shared__ double bred[TR_WARPS][32];
  __shared__ double s_slot;
  const int G = gridDim.x, b = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned *count = bar, *gen = bar + 1;
  double tau_p = 0.0, scale_p = 0.0, e_p = 0.0;
  bool have_p = false;
  for (int c = 0; c < n - 1; ++c) {
    /* ---- A: w and storage of step c-1, column c update, partial ||x||^2 ---- */
    double alpha_p = 0.0, wpc = 0.0;
    if (have_p) {
      alpha_p = -0.5 * tau_p * tau_p * tr_sum_partials(part_dot, G, &s_slot);
      wpc = tau_p * ybuf[c] + alpha_p; /* v_p(c) = 1 */
    }
    {
      const int cnt = n - c, per = (cnt + G - 1) / G;
      const int r0 = c + b * per, r1 = min(n, r0 + per);
      double nrm = 0.0;
      for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        double a = A[(int64_t)c * n + r];
        if (have_p) {
          const double vpr = (r == c) ? 1.0 : A[(int64_t)(c - 1) * n + r] * scale_p;
          const double wpr = tau_p * ybuf[r] + alpha_p * vpr;
          wbuf[r] = wpr;
          A[(int64_t)(c - 1) * n + r] = (r == c) ? e_p : vpr;
          a = a - vpr * wpc - wpr;
        }
        A[(int64_t)c * n + r] = a;
        if (r >= c + 2) nrm = fma(a, a, nrm);
      }
      nrm = tr_block_sum(nrm, red);
      if (threadIdx.x == 0) part_norm[b] = nrm;
    }
    if (!tr_grid_sync(count, gen, err)) return;
    /* ---- reflector of column c (every block, same arithmetic) ---- */
    const double xn2 = tr_sum_partials(part_norm, G, &s_slot);
    const double alpha = A[(int64_t)c * n + c + 1];
    double beta, tau_c, scale_c;
    if (xn2 == 0.0) {
      beta = alpha;
      tau_c = 0.0;
      scale_c = 0.0;
    } else {
      const double xn = sqrt(xn2);
      const double ax = fabs(alpha), big = fmax(ax, xn), sml = fmin(ax, xn);
      const double r = sml / big;
      const double nrm = big * sqrt(1.0 + r * r);
      beta = alpha >= 0.0 ? -nrm : nrm;
      tau_c = (beta - alpha) / beta;
      scale_c = 1.0 / (alpha - beta);
    }
    if (b == 0 && threadIdx.x == 0) {
      d[c] = A[(int64_t)c * n + c];
      e[c] = beta;
      tau[c] = tau_c;
    }
    /* ---- B1: pending update + lower product, warp per column ---- */
    const int m = n - c - 1;
    for (int q = c + 1 + threadIdx.x; q < n; q += blockDim.x) {
      svp[q] = have_p ? A[(int64_t)(c - 1) * n + q] : 0.0;
      swp[q] = have_p ? wbuf[q] : 0.0;
      svc[q] = (q == c + 1) ? 1.0 : A[(int64_t)c * n + q] * scale_c;
    }
    __syncthreads();
    {
      const int u0 = tr_split_cols(m, b, G), u1 = tr_split_cols(m, b + 1, G);
      for (int u = u0 + warp; u < u1; u += TR_WARPS) {
        const int r = c + 1 + u;
        const double vpr = svp[r], wpr = swp[r];
        double *col = A + (int64_t)r * n;
        double dot = 0.0;
        if (have_p) {
          for (int q = r + lane; q < n; q += 32) {
            double a = col[q];
            a = fma(-svp[q], wpr, a);
            a = fma(-swp[q], vpr, a);
            col[q] = a;
            dot = fma(a, svc[q], dot);
          }
        } else {
          for (int q = r + lane; q < n; q += 32) dot = fma(col[q], svc[q], dot);
        }
        for (int o = 16; o; o >>= 1) dot += __shfl_down_sync(0xFFFFFFFFu, dot, o);
        if (lane == 0) ybuf[r] = dot;
      }
    }
    if (!tr_grid_sync(count, gen, err)) return;
    /* ---- B2: strictly lower part of the product, lanes over rows ---- */
    {
      const int u0 = tr_split_rows(m, b, G), u1 = tr_split_rows(m, b + 1, G);
      double dpart = 0.0;
      for (int ch = u0; ch < u1; ch += 32) {
        const int u = ch + lane;
        const int r = c + 1 + u;
        const bool valid = u < u1;
        const int qend = c + 1 + min(ch + 32, u1); /* columns below the chunk's last row */
        double acc = 0.0;
        for (int q = c + 1 + warp; q < qend; q += TR_WARPS)
          if (valid && q < r) acc = fma(A[(int64_t)q * n + r], svc[q], acc);
        bred[warp][lane] = acc;
        __syncthreads();
        if (warp == 0 && valid) {
          double y1 = 0.0;
          for (int w = 0; w < TR_WARPS; ++w) y1 += bred[w][lane];
          const double y = ybuf[r] + y1;
          ybuf[r] = y;
          dpart = fma(y, svc[r], dpart);
        }
        __syncthreads();
      }
      dpart = tr_block_sum(dpart, red);
      if (threadIdx.x == 0) part_dot[b] = dpart;
    }
    if (!tr_grid_sync(count, gen, err)) return;
    tau_p = tau_c;
    scale_p = scale_c;
    e_p = beta;
    have_p = true;
  }
  /* last diagonal entry and the storage of the last reflector */
  if (b == 0) {
    double alpha_p = 0.0;
    if (have_p) alpha_p = -0.5 * tau_p * tau_p * tr_sum_partials(part_dot, G, &s_slot);
    if (threadIdx.x == 0) {
      double a = A[(int64_t)(n - 1) * n + n - 1];
      if (have_p) {
        const double wp = tau_p * ybuf[n - 1] + alpha_p;
        a = a - wp - wp;
        A[(int64_t)(n - 2) * n + n - 1] = e_p;
      }
      d[n - 1] = a;
    }
  }
}

/* deterministic start vector entry in (-1, 1) */
__device__ __forceinline__ double start_entry(int j, int i)
{
  uint64_t z = ((uint64_t)(j + 1) << 32) ^ (uint64_t)(i + 1) ^ 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return ((double)(z >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

__device__ double block_sum(double v, double *red)
{
  red[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

/*
 * Inverse iteration, one block per top eigenvalue (vector j belongs to w[n-1-j]).
 * The LU factorisation with partial pivoting of T - lam I and the solves are sequential
 * recurrences run by thread 0 with the running values carried in registers (the arrays are
 * only written, or read ahead of the dependency chain); the other threads normalise.
 * work: per vector 6n doubles.  Z [nvec][n] (column-major N x nvec for ormtr).
 */
__global__ void k_inverse_iteration(const double *d, const double *e, int n, const double *w,
                                    int nvec, double tnorm, double *Z, double *work)
{
  __shared__ double red[256];
  const int j = blockIdx.x;
  if (j >= nvec) return;
  double *base = work + (int64_t)j * 6 * n;
  double *Dinv = base, *DL = base + n, *DU = base + 2 * n, *DU2 = base + 3 * n;
  double *x = Z + (int64_t)j * n;
  int *piv = (int *)(base + 5 * n);
  const double lam = w[n - 1 - j];
  const double tiny = DBL_EPSILON * tnorm;
  if (threadIdx.x == 0) {
    /* dgttrf-style elimination; cur = running diagonal of row i, du = its superdiagonal */
    double cur = d[0] - lam;
    double du = n > 1 ? e[0] : 0.0;
    for (int i = 0; i < n - 1; ++i) {
      double ei = e[i];
      double dn = d[i + 1] - lam;                    /* row i+1 diagonal */
      double en = (i < n - 2) ? e[i + 1] : 0.0;      /* row i+1 superdiagonal */
      if (fabs(cur) >= fabs(ei)) {
        if (cur == 0.0) cur = tiny;
        double f = ei / cur;
        DL[i] = f;
        DU[i] = du;
        DU2[i] = 0.0;
        Dinv[i] = 1.0 / cur;
        piv[i] = 0;
        cur = dn - f * du;
        du = en;
      } else {
        double f = cur / ei;
        DL[i] = f;
        Dinv[i] = 1.0 / ei;
        DU[i] = dn;
        DU2[i] = en;
        piv[i] = 1;
        cur = du - f * dn;
        du = -f * en;
      }
    }
    if (cur == 0.0) cur = tiny;
    Dinv[n - 1] = 1.0 / cur;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = start_entry(j, i);
  __syncthreads();
  for (int iter = 0; iter < 3; ++iter) {
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s2 += x[i] * x[i];
    s2 = block_sum(s2, red);
    double inv = s2 > 0.0 ? 1.0 / sqrt(s2) : 1.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] *= inv;
    __syncthreads();
    if (threadIdx.x == 0) {
      /* forward: apply the row interchanges and L; carry x[i+1] in a register */
      double xi = x[0];
      for (int i = 0; i < n - 1; ++i) {
        double xn = x[i + 1];
        if (piv[i] == 0) {
          x[i] = xi;
          xi = xn - DL[i] * xi;
        } else {
          x[i] = xn;
          xi = xi - DL[i] * xn;
        }
      }
      x[n - 1] = xi;
      /* back substitution with U (diag, super, super-super) */
      double x2 = 0.0, x1 = x[n - 1] * Dinv[n - 1];
      x[n - 1] = x1;
      for (int i = n - 2; i >= 0; --i) {
        double v = (x[i] - DU[i] * x1 - DU2[i] * x2) * Dinv[i];
        x[i] = v;
        x2 = x1;
        x1 = v;
      }
    }
    __syncthreads();
  }
  double s2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s2 += x[i] * x[i];
  s2 = block_sum(s2, red);
  double inv = 1.0 / sqrt(s2);
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] *= inv;
}

/* modified Gram-Schmidt over the nvec vectors, in order (one block) */
__global__ void k_mgs(double *Z, int n, int nvec)
{
  __shared__ double red[256];
  for (int j = 0; j < nvec; ++j) {
    double *zj = Z + (int64_t)j * n;
    for (int p = 0; p < j; ++p) {
      const double *zp = Z + (int64_t)p * n;
      double s = 0.0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) s += zp[i] * zj[i];
      s = block_sum(s, red);
      for (int i = threadIdx.x; i < n; i += blockDim.x) zj[i] -= s * zp[i];
      __syncthreads();
    }
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s2 += zj[i] * zj[i];
    s2 = block_sum(s2, red);
    double inv = 1.0 / sqrt(s2);
    for (int i = threadIdx.x; i < n; i += blockDim.x) zj[i] *= inv;
    __syncthreads();
  }
}

/* evals_desc[i] = w[n-1-i] */
__global__ void k_reverse(const double *w, double *out, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = w[n - 1 - i];
}

/*
 * Eigenpairs of the symmetric n x n matrix in ctx->d_xtx (overwritten): d_evals_desc [n]
 * all eigenvalues descending, d_vecs [nvec][n] top eigenvectors (descending).
 */
int gp_eig_tridiag(gp_ctx *ctx, int32_t n, int32_t nvec, double *d_evals_desc, double *d_vecs)
{
  cusolverDnHandle_t h = ctx->solver;
  int lwork = 0, lwork2 = 0;
  /* GP_EIG_TIMING=1 prints the device time of each stage to stderr */
  const char *tenv = getenv("GP_EIG_TIMING");
  const int timing = tenv && tenv[0] == '1';
  cudaEvent_t ev[5];
  if (timing)
    for (int i = 0; i < 5; ++i) cudaEventCreate(&ev[i]);
#define GP_EIG_MARK(i) \
  if (timing) cudaEventRecord(ev[i], ctx->stream)
  /* scratch: d, e, tau, e2, w, work(sytrd), inverse-iteration work, info */
  if (cusolverDnDsytrd_bufferSize(h, CUBLAS_FILL_MODE_LOWER, n, ctx->d_xtx, n, NULL, NULL, NULL,
                                  &lwork) != CUSOLVER_STATUS_SUCCESS)
    return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDsytrd_bufferSize failed");
  int nv = nvec > 0 ? nvec : 1;
  if (cusolverDnDormtr_bufferSize(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, nv,
                                  ctx->d_xtx, n, NULL, d_vecs, n, &lwork2) != CUSOLVER_STATUS_SUCCESS)
    return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDormtr_bufferSize failed");
  int lw = lwork > lwork2 ? lwork : lwork2;
  size_t nd = (size_t)n;
  size_t bytes = sizeof(double) * (5 * nd + (size_t)lw + 6 * nd * nv + 64) + sizeof(int) * 64;
  double *base;
  int rc = gp_scratch(ctx, bytes, (void **)&base);
  if (rc) return rc;
  double *d = base, *e = d + nd, *tau = e + nd, *e2 = tau + nd, *w = e2 + nd;
  double *ws = w + nd, *iw = ws + lw;
  int *d_info = (int *)(iw + 6 * nd * nv + 8);
  GP_EIG_MARK(0);
  if (cusolverDnDsytrd(h, CUBLAS_FILL_MODE_LOWER, n, ctx->d_xtx, n, d, e, tau, ws, lw, d_info) !=
      CUSOLVER_STATUS_SUCCESS)
    return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDsytrd failed to launch");
  GP_EIG_MARK(1);
  int info = 0;
  GP_CUDA(ctx, gp_memcpy(ctx, &info, d_info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  /* Gershgorin bounds and the pivot guard need d, e on the host (2n doubles) */
  std::vector<double> hd(nd), he(nd > 1 ? nd - 1 : 1);
  GP_CUDA(ctx, gp_memcpy(ctx, hd.data(), d, sizeof(double) * nd, cudaMemcpyDeviceToHost, ctx->stream));
  if (n > 1)
    GP_CUDA(ctx, gp_memcpy(ctx, he.data(), e, sizeof(double) * (nd - 1), cudaMemcpyDeviceToHost,
                           ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (info != 0) return gp_fail(ctx, GP_ERR_SOLVER, "sytrd info = %d", info);
  double gl = hd[0], gu = hd[0], tnorm = 0.0, emax2 = 0.0;
  std::vector<double> he2(nd > 1 ? nd - 1 : 1);
  for (int i = 0; i < n; ++i) {
    double r = (i > 0 ? fabs(he[(size_t)i - 1]) : 0.0) + (i < n - 1 ? fabs(he[(size_t)i]) : 0.0);
    gl = fmin(gl, hd[(size_t)i] - r);
    gu = fmax(gu, hd[(size_t)i] + r);
    tnorm = fmax(tnorm, fabs(hd[(size_t)i]) + r);
    if (i < n - 1) {
      he2[(size_t)i] = he[(size_t)i] * he[(size_t)i];
      emax2 = fmax(emax2, he2[(size_t)i]);
    }
  }
  double span = gu - gl;
  gl -= 2.0 * DBL_EPSILON * tnorm * n + DBL_MIN;
  gu += 2.0 * DBL_EPSILON * tnorm * n + DBL_MIN;
  (void)span;
  /* the pivot guard stays inside FP32's exponent range (the reciprocal starts in FP32) */
  double pivmin = fmax(DBL_MIN * fmax(1.0, emax2), 1e-30 * fmax(tnorm, 1e-300));
  if (n > 1)
    GP_CUDA(ctx, gp_memcpy(ctx, e2, he2.data(), sizeof(double) * (nd - 1), cudaMemcpyHostToDevice,
                           ctx->stream));
  GP_EIG_MARK(2);
  {
    size_t smem = (size_t)24 * (size_t)n;
    int use_smem = smem <= 200 * 1024;
    const int warps = ctx->num_sms * 4;
    int epw = (n + warps - 1) / warps;
    if (epw > 32) epw = 32;
    const int P = 32 / epw;
    const int nwarps = (n + epw - 1) / epw;
    const int blocks = (nwarps + 3) / 4;
    /* FP64 brackets end at 1e-13 ||T||: the counts' own backward error is ~6e-14 ||T|| */
    const double tol = 1e-13 * tnorm;
    if (use_smem)
      GP_CUDA(ctx, cudaFuncSetAttribute(k_multisect, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
    k_multisect<<<blocks, 128, use_smem ? smem : 0, ctx->stream>>>(d, e2, n, gl, gu, tnorm, pivmin,
                                                                   tol, use_smem, epw, P, w);
    GP_LAUNCH_CHECK(ctx, "k_multisect");
  }
  k_reverse<<<(n + 255) / 256, 256, 0, ctx->stream>>>(w, d_evals_desc, n);
  GP_LAUNCH_CHECK(ctx, "k_reverse");
  GP_EIG_MARK(3);
  if (nvec > 0) {
    k_inverse_iteration<<<nvec, 256, 0, ctx->stream>>>(d, e, n, w, nvec, tnorm, d_vecs, iw);
    GP_LAUNCH_CHECK(ctx, "k_inverse_iteration");
    k_mgs<<<1, 256, 0, ctx->stream>>>(d_vecs, n, nvec);
    GP_LAUNCH_CHECK(ctx, "k_mgs");
    if (cusolverDnDormtr(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, nvec,
                         ctx->d_xtx, n, tau, d_vecs, n, ws, lw, d_info) != CUSOLVER_STATUS_SUCCESS)
      return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDormtr failed to launch");
    GP_CUDA(ctx, gp_memcpy(ctx, &info, d_info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (info != 0) return gp_fail(ctx, GP_ERR_SOLVER, "ormtr info = %d", info);
  }
  if (timing) {
    GP_EIG_MARK(4);
    cudaEventSynchronize(ev[4]);
    float t01 = 0, t23 = 0, t34 = 0;
    cudaEventElapsedTime(&t01, ev[0], ev[1]);
    cudaEventElapsedTime(&t23, ev[2], ev[3]);
    cudaEventElapsedTime(&t34, ev[3], ev[4]);
    fprintf(stderr, "eig n=%d: sytrd %.1f ms, eigenvalues %.1f ms, vectors+ormtr %.1f ms\n", n,
            t01, t23, t34);
    for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
  }
  return GP_OK;
}
