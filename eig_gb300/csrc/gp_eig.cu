/*
 * Dense symmetric FP64 eigensolve for the smartpca Gram, on the device: all N eigenvalues
 * and the top nvec eigenvectors (the reference computes every eigenpair with LAPACK dspev,
 * src/eigensrc/eigx.c:97-117, but prints all eigenvalues and uses only the top vectors).
 *
 *   1. Householder tridiagonalisation A = Q T Q^T (k_tridiag below: one cooperative launch,
 *      LAPACK dsytd2's reflectors and storage; cuSOLVER sytrd beyond 8,533 rows);
 *   2. all eigenvalues of T by multisection on Sturm counts (the published bisection method:
 *      the count of negative pivots of the LDL^T factorisation of T - x I equals the number
 *      of eigenvalues below x), several lanes per eigenvalue index: FP32 brackets first,
 *      then float-float, checked and finished in FP64 to 1e-13 ||T||;
 *   3. the top nvec eigenvectors of T by inverse iteration, one block per vector: LU with
 *      partial pivoting of the tridiagonal T - lambda I (Gaussian elimination with row
 *      interchanges) and three solves from a fixed pseudo-random start, then modified
 *      Gram-Schmidt over the vectors in order (eigenvalues that are distinct to far more than
 *      eps*||T|| make each iterate converge to its own eigenvector);
 *   4. back-transformation of those nvec vectors only, V = Q Z (k_apply_q: compact WY blocks
 *      of 32 reflectors in float-float; cuSOLVER ormtr when its row slab does not fit).
 */
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <float.h>
#include <algorithm>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "gp_internal.h"
#include "gp_tc.cuh"


/*
 * Float-float arithmetic: a value is an unevaluated sum h + l of two FP32 numbers (about 46
 * significant bits), built from the error-free transformations TwoSum (Knuth) and TwoProd
 * with FMA (Dekker / Ogita-Rump-Oishi 2005).  GB300's FP64 pipe issues about 2 FMAs per clock
 * per SM and its FP32 pipe 128, so the tridiagonalisation keeps its trailing matrix and
 * vectors in this form; every operation below is explicitly rounded (no contraction).
 */
struct ff2 {
  float h, l;
};

__device__ __forceinline__ ff2 ff_make(float h, float l)
{
  ff2 r;
  r.h = h;
  r.l = l;
  return r;
}
__device__ __forceinline__ ff2 ff_from_double(double x)
{
  const float h = __double2float_rn(x);
  return ff_make(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double ff_to_double(ff2 a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ ff2 ff_neg(ff2 a) { return ff_make(-a.h, -a.l); }
/* a + b */
__device__ __forceinline__ ff2 ff_add(ff2 a, ff2 b)
{
  const float s = __fadd_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  err = __fadd_rn(err, __fadd_rn(a.l, b.l));
  const float h = __fadd_rn(s, err);
  return ff_make(h, __fsub_rn(err, __fsub_rn(h, s)));
}
/* a * b */
__device__ __forceinline__ ff2 ff_mul(ff2 a, ff2 b)
{
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  const float h = __fadd_rn(p, e);
  return ff_make(h, __fsub_rn(e, __fsub_rn(h, p)));
}
/* a * b + c */
__device__ __forceinline__ ff2 ff_fma(ff2 a, ff2 b, ff2 c)
{
  const float p = __fmul_rn(a.h, b.h);
  float pe = __fmaf_rn(a.h, b.h, -p);
  pe = __fmaf_rn(a.h, b.l, pe);
  pe = __fmaf_rn(a.l, b.h, pe);
  const float s = __fadd_rn(c.h, p);
  const float bb = __fsub_rn(s, c.h);
  float err = __fadd_rn(__fsub_rn(c.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  err = __fadd_rn(err, __fadd_rn(c.l, pe));
  const float h = __fadd_rn(s, err);
  return ff_make(h, __fsub_rn(err, __fsub_rn(h, s)));
}
__device__ __forceinline__ ff2 ff_shfl_xor(ff2 a, int o)
{
  return ff_make(__shfl_xor_sync(0xFFFFFFFFu, a.h, o), __shfl_xor_sync(0xFFFFFFFFu, a.l, o));
}
__device__ __forceinline__ ff2 ff_load(const double *p)
{
  const float2 v = *reinterpret_cast<const float2 *>(p);
  return ff_make(v.x, v.y);
}
__device__ __forceinline__ void ff_store(double *p, ff2 a)
{
  *reinterpret_cast<float2 *>(p) = make_float2(a.h, a.l);
}

/* sqrt(a) for a > 0: FP32 root plus one correction, (a - s^2) / 2s */
__device__ __forceinline__ ff2 ff_sqrt(ff2 a)
{
  const float s = sqrtf(a.h);
  const ff2 r = ff_fma(ff_make(-s, 0.f), ff_make(s, 0.f), a);
  return ff_add(ff_make(s, 0.f), ff_make(__fdiv_rn(r.h, 2.f * s), 0.f));
}
/* a / b: FP32 quotient plus one correction from the float-float remainder */
__device__ __forceinline__ ff2 ff_div(ff2 a, ff2 b)
{
  const float q1 = __fdiv_rn(a.h, b.h);
  const ff2 r = ff_fma(ff_neg(b), ff_make(q1, 0.f), a);
  return ff_add(ff_make(q1, 0.f), ff_make(__fdiv_rn(r.h, b.h), 0.f));
}
__device__ __forceinline__ ff2 ff_scale(ff2 a, float s) { return ff_make(a.h * s, a.l * s); }

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

/* a / b in float-float from the FP32 approximate reciprocal and one remainder correction
 * (relative error ~2^-44; the Sturm brackets below allow for it) */
__device__ __forceinline__ ff2 ff_div_approx(ff2 a, ff2 b)
{
  float rb;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(b.h));
  const float q1 = __fmul_rn(a.h, rb);
  const ff2 r = ff_fma(ff_neg(b), ff_make(q1, 0.f), a);
  const float q2 = __fmul_rn(r.h, rb);
  const float h = __fadd_rn(q1, q2);
  return ff_make(h, __fsub_rn(q2, __fsub_rn(h, q1)));
}

/* the Sturm count in float-float (d and e2 as hi/lo FP32 pairs; verified in FP64 afterwards) */
__device__ __forceinline__ int sturm_count_ff(const float *dh, const float *dl, const float *eh,
                                              const float *el, int n, ff2 x, float pivmin)
{
  const ff2 nx = ff_neg(x), clamp = ff_make(-pivmin, 0.f);
  ff2 q = ff_add(ff_make(dh[0], dl[0]), nx);
  if (fabsf(q.h) < pivmin) q = clamp;
  int cnt = q.h < 0.f;
  for (int i = 1; i < n; ++i) {
    const ff2 t = ff_add(ff_make(dh[i], dl[i]), nx);
    q = ff_add(t, ff_neg(ff_div_approx(ff_make(eh[i - 1], el[i - 1]), q)));
    if (fabsf(q.h) < pivmin) q = clamp;
    cnt += q.h < 0.f;
  }
  return cnt;
}

/*
 * All eigenvalues by multisection: a warp owns epw consecutive eigenvalue indices and each
 * index gets P = 32/epw lanes (P >= 1), so every warp slot of the GPU has work whatever N is.
 * A step evaluates P interior points of the bracket at once (one Sturm count per lane) and
 * keeps the sub-interval where the count crosses k: log2(P+1) bits per step.  FP32 counts
 * narrow the bracket to ~4e-7 ||T|| (widened by 64 eps_32 ||T||), float-float counts on the
 * FP32 pipe narrow it to ~1e-12 ||T|| (widened by 64 2^-44 ||T||), two FP64 counts check it
 * (back to the Gershgorin bracket if the check fails), then FP64 counts narrow it to tol.
 * Grid: one CTA of 4 warps per SM; d, e2 and their FP32 hi/lo copies in shared memory
 * (32 N bytes) when they fit (use_smem 2), d, e2 and FP32 copies without the float-float
 * phase (24 N bytes, use_smem 1), else FP64 counts from global memory only.
 */
__global__ void __launch_bounds__(128)
k_multisect(const double *gd, const double *ge2, int n, double gl, double gu, double tnorm,
            double pivmin, double tol, int use_smem, int epw, int P, double *w)
{
  extern __shared__ double sm[];
  const double *d = gd, *e2 = ge2;
  const float *df = NULL, *e2f = NULL, *dl = NULL, *e2l = NULL;
  if (use_smem) {
    double *sd = sm, *se2 = sm + n;
    float *sdf = (float *)(sm + 2 * n), *se2f = sdf + n;
    float *sdl = se2f + n, *se2l = sdl + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      sd[i] = gd[i];
      sdf[i] = (float)gd[i];
      if (use_smem > 1) sdl[i] = (float)(gd[i] - (double)sdf[i]);
      if (i < n - 1) {
        se2[i] = ge2[i];
        se2f[i] = (float)ge2[i];
        if (use_smem > 1) se2l[i] = (float)(ge2[i] - (double)se2f[i]);
      }
    }
    __syncthreads();
    d = sd;
    e2 = se2;
    df = sdf;
    e2f = se2f;
    if (use_smem > 1) {
      dl = sdl;
      e2l = se2l;
    }
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
    if (dl) {
      /* float-float phase: the same multisection with x_j = lo + (hi - lo) j / (P+1) formed
       * identically for a point and for the bracket end it becomes */
      ff2 glo = ff_from_double(lo), ghi = ff_from_double(hi);
      const float fpiv = fmaxf((float)pivmin, 1e-30f);
      const float ftol2 = (float)(1e-12 * tnorm);
      for (int it = 0; it < 64; ++it) {
        const ff2 wdt = ff_add(ghi, ff_neg(glo));
        if (!(wdt.h > ftol2)) break;
        const ff2 x = ff_fma(wdt, ff_make((float)(sub + 1) / (float)(P + 1), 0.f), glo);
        const bool inside = ff_add(x, ff_neg(glo)).h > 0.f && ff_add(ghi, ff_neg(x)).h > 0.f;
        const int flag = inside ? (sturm_count_ff(df, dl, e2f, e2l, n, x, fpiv) > k)
                                : (ff_add(x, ff_neg(ghi)).h >= 0.f);
        const unsigned b = (__ballot_sync(gmask, flag) >> gshift) & gbits;
        const int first = b ? __ffs(b) - 1 : P;
        const ff2 nlo =
            first == 0 ? glo : ff_fma(wdt, ff_make((float)first / (float)(P + 1), 0.f), glo);
        const ff2 nhi =
            first == P ? ghi : ff_fma(wdt, ff_make((float)(first + 1) / (float)(P + 1), 0.f), glo);
        if (!(ff_add(nhi, ff_neg(nlo)).h < wdt.h)) break;
        glo = nlo;
        ghi = nhi;
      }
      const double margin2 = 64.0 * 0x1p-44 * tnorm;
      lo = fmax(gl, ff_to_double(glo) - margin2);
      hi = fmin(gu, ff_to_double(ghi) + margin2);
    }
    int ok = 1;
    if (sub < 2) {
      const double x = sub == 0 ? lo : hi;
      const int c = sturm_count_bits(d, e2, n, x, pivmin);
      ok = sub == 0 ? (c <= k) : (c > k);
      if (P == 1) ok = ok && sturm_count_bits(d, e2, n, hi, pivmin) > k; /* one lane: both ends */
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
 * Householder tridiagonalisation A = Q T Q^T of the symmetric n x n matrix (held in full,
 * column-major: element (r, q) at A[q*n + r]), the unblocked algorithm of LAPACK dsytd2
 * (lower) restated for one cooperative launch:
 *   for c = 0 .. n-2:  x = A(c+1:n, c);  (beta, tau, v) = reflector of x (dlarfg: v(c+1) = 1,
 *   beta = -sign(alpha) ||x||, tau = (beta - alpha)/beta, v = x/(alpha - beta) below);
 *   y = A(c+1:n, c+1:n) v;  w = tau y - (tau^2/2)(y.v) v;  A(c+1:n, c+1:n) -= v w^T + w v^T.
 * The rank-2 update of step c is not a pass of its own: it is applied while step c+1 reads the
 * trailing matrix for its product (look-ahead).  Both triangles of the trailing matrix are
 * kept up to date, so the product is a dot of each whole column with v: every block owns an
 * even share of the columns (equal lengths), reads and writes them once, and no block needs
 * another block's columns within the step.  Per step:
 *   A   every block rebuilds, from y and x of step c-1 and column c, the vectors v and w of
 *       step c-1, the pending update of column c, its norm and the reflector (O(n) work done
 *       redundantly instead of a grid-wide reduction); each block writes its share of the
 *       reflector storage of step c-1 (LAPACK's, e(c-1) on the subdiagonal) and of x_c
 *   B   each block, per owned column r: pending update of A(c+1:n, r), written back, and
 *       y(r) = A(c+1:n, r) . v, warp per column (segments when the block has fewer columns
 *       than warps); then its share of y . v
 *   --- grid barrier
 * x and y are double-buffered across steps, so phase A of one step never reads a vector
 * that a faster block is already writing in the next.
 * Every sum has a fixed order (no atomics), so the result is deterministic.  The grid
 * barrier is a monotonic counter with a %globaltimer bound: on expiry the kernel records an
 * error code and returns (the host reports GP_ERR_TIMEOUT).
 * Outputs: d[n], e[n-1], tau[n-1] and the reflectors in the lower triangle of A, as
 * dormtr (lower) reads them.  Shared memory: v(step c-1), w(step c-1), v(step c) over the
 * rows (24 n bytes).
 */
#define TR_THREADS 1024
#define TR_WARPS (TR_THREADS / 32)
#define TR_U 8 /* loads in flight per lane in the product loops */
#define TR_B1_SLOTS 256 /* segment dots of one block in the column pass */
#define TR_ERR_BARRIER 11

/* arrival with release semantics at GPU scope (the block's writes, ordered before it by the
 * block barrier, become visible to a block that acquires the count) */
__device__ __forceinline__ void red_release_gpu(unsigned *p, unsigned v)
{
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p)
{
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

/* grid barrier on a monotonic arrival counter: the k-th barrier of the launch waits until
 * k * gridDim.x blocks have arrived (one release-add per block, acquire loads while
 * waiting, no reset) */
__device__ __forceinline__ bool tr_grid_sync(unsigned *count, unsigned target, int *err)
{
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile int *verr = err;
    red_release_gpu(count, 1u);
    const uint64_t t0 = globaltimer_ns();
    for (unsigned it = 1; ld_acquire_gpu(count) < target; ++it) {
      if ((it & 63u) == 0) {
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

/* sum of the G float-float block partials in a fixed order (warp 0), broadcast */
__device__ __forceinline__ ff2 ff_sum_partials(const double *part, int G, ff2 *slot)
{
  if (threadIdx.x < 32) {
    ff2 s = ff_make(0.f, 0.f);
    for (int g = threadIdx.x; g < G; g += 32) s = ff_add(s, ff_load(part + g));
    for (int o = 16; o; o >>= 1) s = ff_add(s, ff_shfl_xor(s, o));
    if (threadIdx.x == 0) *slot = s;
  }
  __syncthreads();
  const ff2 r = *slot;
  __syncthreads();
  return r;
}

/* block sum of one float-float per thread (fixed order: warp shuffles, then warp 0's
 * shuffle tree over the warps' sums), as float-float in thread 0 */
__device__ __forceinline__ ff2 ff_block_sum2(ff2 v, ff2 *red)
{
  static_assert(TR_WARPS == 32, "one warp sums the warps' partials");
  for (int o = 16; o; o >>= 1) v = ff_add(v, ff_shfl_xor(v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  ff2 t = ff_make(0.f, 0.f);
  if (threadIdx.x < 32) {
    t = red[threadIdx.x];
    for (int o = 16; o; o >>= 1) t = ff_add(t, ff_shfl_xor(t, o));
  }
  __syncthreads();
  return t;
}

/* block sum of one float-float per thread (fixed order), as a double in thread 0 */
__device__ __forceinline__ double ff_block_sum(ff2 v, ff2 *red)
{
  for (int o = 16; o; o >>= 1) v = ff_add(v, ff_shfl_xor(v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    ff2 t = red[0];
    for (int w = 1; w < TR_WARPS; ++w) t = ff_add(t, red[w]);
    s = ff_to_double(t);
  }
  __syncthreads();
  return s;
}

/* the (symmetric, full) double matrix to float-float pairs, in place */
__global__ void k_tri_to_ff(double *A, int n)
{
  const int64_t total = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x)
    ff_store(A + idx, ff_from_double(A[idx]));
}

/* per-step scalars, computed once per block by thread 0 (GB300's FP64 pipe is narrow, so
 * scalar square roots and divisions are not repeated by every thread) */
struct tr_step {
  ff2 beta, tau_c, scale_c;
  int b1_u0, b1_u1;
};

/*
 * A holds the whole matrix as float-float pairs on entry (k_tri_to_ff); vbuf/wbuf hold the
 * updated column x of alternate steps, ybuf [2n] the product y of alternate steps and
 * part_dot2 [2G] the blocks' partial y.v of alternate steps, as float-float pairs in doubles'
 * storage.  On exit the reflectors are FP64 again in A(c+2:n, c) and e on the subdiagonal, as
 * dormtr (lower) reads them; the upper triangle is left in float-float form.
 */
/*
 * Steps c_begin .. n-2 of the whole-matrix reduction (k_tridiag's step; the tail steps of
 * k_tridiag_tiled): A holds the trailing matrix (indices >= c_begin) as float-float pairs in
 * whole columns, both triangles.  svp/swp/svc: the block's vectors in shared memory (at least
 * n pairs each).  tau_pf, scale_pf, e_pf, have_p and target carry the previous step's state.
 * dot0 (when not NULL) holds the previous step's y.v parts at [dot0_k0, dot0_k1) instead of
 * part_dot2 (the step before c_begin was a tiled one).  sph (block 0, thread 0 only; else
 * NULL): phase times as in k_tridiag, sph[5] the last time stamp.  False when the grid
 * barrier failed.
 */
__device__ __forceinline__ bool tr_full_steps(double *A, int n, int c_begin, double *d, double *e,
                                              double *tau, double *vbuf, double *wbuf,
                                              double *ybuf, double *part_dot2, unsigned *count,
                                              unsigned &target, int *err, double *svp,
                                              double *swp, double *svc, ff2 &tau_pf,
                                              ff2 &scale_pf, ff2 &e_pf, bool &have_p,
                                              const double *dot0, int dot0_k0, int dot0_k1,
                                              unsigned long long *sph)
{
  __shared__ ff2 red[TR_WARPS];
  __shared__ ff2 sdotp[TR_B1_SLOTS];
  __shared__ tr_step st;
  __shared__ ff2 s_slotf;
  const int G = gridDim.x, b = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const ff2 ONE = ff_make(1.f, 0.f), ZERO = ff_make(0.f, 0.f);
  const bool stamp = sph != NULL;
#define TR_STAMP(i)                                    \
  if (stamp) {                                         \
    const unsigned long long t_now = globaltimer_ns(); \
    sph[i] += t_now - sph[5];                          \
    sph[5] = t_now;                                    \
  }
  const int early = (int)((3LL * n) / 10);
  for (int c = c_begin; c < n - 1; ++c) {
    /* ---- A (every block, no grid barrier): v and w of step c-1, the pending update of
     * column c and its norm, rebuilt from y, the stored x of step c-1 and column c; each
     * block also writes its share of the reflector storage and of x_c (double buffer) ---- */
    const int m = n - c - 1;
    double *xcur = (c & 1) ? wbuf : vbuf, *xprev = (c & 1) ? vbuf : wbuf;
    /* y of step c and of step c-1 (double buffer: phase A reads one while B writes the other) */
    double *ycur = ybuf + (int64_t)(c & 1) * n, *yprev = ybuf + (int64_t)((c + 1) & 1) * n;
    if (threadIdx.x == 32) st.b1_u0 = (int)(((int64_t)m * b) / G);
    if (threadIdx.x == 33) st.b1_u1 = (int)(((int64_t)m * (b + 1)) / G);
    /* the block partials of y.v of step c-1 (double buffer: blocks already in step c+1 write
     * the other half), loaded by the last warp ahead of the vector loads so that the two
     * latencies overlap; summed per lane in order, then by a fixed shuffle tree */
    ff2 pacc = ZERO;
    if (have_p && warp == TR_WARPS - 1) {
      const double *pprev = part_dot2 + (size_t)((c + 1) & 1) * G;
      int g0 = 0, g1 = G;
      if (c == c_begin && dot0 != NULL) { /* the previous step was a tiled one */
        pprev = dot0;
        g0 = dot0_k0;
        g1 = dot0_k1;
      }
#pragma unroll 4
      for (int g = g0 + lane; g < g1; g += 32) pacc = ff_add(pacc, ff_load(pprev + g));
    }
    /* loads (v_p needs only step c-1's scale; y is kept raw in swp for now) */
#pragma unroll 4
    for (int q = c + threadIdx.x; q < n; q += blockDim.x) {
      ff2 vp = ZERO, yq = ZERO;
      if (have_p) {
        vp = (q == c) ? ONE : ff_mul(ff_load(xprev + q), scale_pf);
        yq = ff_load(yprev + q);
      }
      ff_store(svp + q, vp);
      ff_store(swp + q, yq);
      ff_store(svc + q, ff_load(A + (int64_t)c * n + q));
    }
    if (have_p && warp == TR_WARPS - 1) {
      for (int o = 16; o; o >>= 1) pacc = ff_add(pacc, ff_shfl_xor(pacc, o));
      if (lane == 0) s_slotf = pacc;
    }
    __syncthreads(); /* publishes the partial sum and svp, swp, svc */
    ff2 wpc = ZERO, alpha_pf = ZERO;
    if (have_p) {
      /* every thread forms alpha and w_p(c) of step c-1 from the same values */
      const ff2 dsum = s_slotf;
      alpha_pf = ff_scale(ff_mul(ff_mul(tau_pf, tau_pf), dsum), -0.5f);
      wpc = ff_fma(tau_pf, ff_load(swp + c), alpha_pf); /* w_p(c); v_p(c) = 1 */
    }
    {
      const int cnt = n - c, per = (cnt + G - 1) / G;
      const int r0 = c + b * per, r1 = min(n, r0 + per);
      ff2 nrm = ZERO;
      for (int q = c + threadIdx.x; q < n; q += blockDim.x) {
        ff2 x = ff_load(svc + q);
        const bool mine = q >= r0 && q < r1;
        if (have_p) {
          const ff2 vp = ff_load(svp + q);
          const ff2 wp = ff_fma(tau_pf, ff_load(swp + q), ff_mul(alpha_pf, vp));
          ff_store(swp + q, wp);
          x = ff_fma(ff_neg(vp), wpc, x);
          x = ff_add(x, ff_neg(wp));
          if (mine) A[(int64_t)(c - 1) * n + q] = ff_to_double(q == c ? e_pf : vp); /* FP64 */
        }
        ff_store(svc + q, x);
        if (mine) ff_store(xcur + q, x);
        if (q >= c + 2) nrm = ff_fma(x, x, nrm);
      }
      const ff2 xn2 = ff_block_sum2(nrm, red); /* thread 0; the sum's barriers publish svc */
      if (threadIdx.x == 0) {
        /* the reflector (dlarfg) in float-float: beta = -sign(alpha) sqrt(alpha^2 + |x|^2),
         * tau = (beta - alpha) / beta, scale = 1 / (alpha - beta) */
        const ff2 alpha = ff_load(svc + c + 1);
        if (xn2.h == 0.f) {
          st.beta = alpha;
          st.tau_c = ZERO;
          st.scale_c = ZERO;
        } else {
          const ff2 nrm2 = ff_sqrt(ff_fma(alpha, alpha, xn2));
          const ff2 beta = alpha.h >= 0.f ? ff_neg(nrm2) : nrm2;
          const ff2 am = ff_add(alpha, ff_neg(beta));
          st.beta = beta;
          st.tau_c = ff_div(ff_neg(am), beta);
          st.scale_c = ff_div(ONE, am);
        }
      }
      __syncthreads();
      if (b == 0 && threadIdx.x == 32) {
        d[c] = ff_to_double(ff_load(svc + c));
        e[c] = ff_to_double(st.beta);
        tau[c] = ff_to_double(st.tau_c);
      }
    }
    const ff2 beta = st.beta, tau_c = st.tau_c;
    const ff2 scale_cf = st.scale_c;
    TR_STAMP(0)
    /* ---- B: pending update + product over whole columns (both triangles are stored),
     * warp per column; the block's columns are an even share of the trailing matrix ---- */
    for (int q = c + 1 + threadIdx.x; q < n; q += blockDim.x)
      ff_store(svc + q, (q == c + 1) ? ONE : ff_mul(ff_load(svc + q), scale_cf));
    __syncthreads();
    {
      const int u0 = st.b1_u0, u1 = st.b1_u1, ncol = u1 - u0;
      /* one piece [qs, qe) of column r: pending update, store and dot with v; the last
       * partial batch is one predicated round of loads, so no piece ends in a chain of
       * dependent single loads */
      auto piece = [&](int r, int qs, int qe) -> ff2 {
        const ff2 vpr = ff_neg(ff_load(svp + r)), wpr = ff_neg(ff_load(swp + r));
        double *col = A + (int64_t)r * n;
        ff2 dot = ZERO;
        for (int qb = qs; qb < qe; qb += 32 * TR_U) {
          ff2 a[TR_U];
#pragma unroll
          for (int u = 0; u < TR_U; ++u) {
            const int qq = qb + lane + 32 * u;
            a[u] = qq < qe ? ff_load(col + qq) : ZERO;
          }
#pragma unroll
          for (int u = 0; u < TR_U; ++u) {
            const int qq = qb + lane + 32 * u;
            if (qq < qe) {
              if (have_p) {
                a[u] = ff_fma(ff_load(svp + qq), wpr, a[u]);
                a[u] = ff_fma(ff_load(swp + qq), vpr, a[u]);
                ff_store(col + qq, a[u]);
              }
              dot = ff_fma(a[u], ff_load(svc + qq), dot);
            }
          }
        }
        for (int o = 16; o; o >>= 1) dot = ff_add(dot, ff_shfl_xor(dot, o));
        return dot;
      };
      /* work items (column, segment): a block with fewer columns than warps splits each into
       * S segments so that every warp works; segment dots are summed in order.  (Equal
       * flattened element ranges per warp measured slower than this split.) */
      const int S = (ncol > 0 && ncol < TR_WARPS) ? (TR_WARPS + ncol - 1) / ncol : 1;
      const int nitem = ncol * S;
      const int seg = ((m + S - 1) / S + 31) & ~31;
      for (int it = warp; it < nitem; it += TR_WARPS) {
        const int j = it / S, sg = it - j * S;
        const int qs = c + 1 + sg * seg, qe = min(n, qs + seg);
        const ff2 dot = piece(c + 1 + u0 + j, qs, qe);
        if (lane == 0) {
          if (S == 1)
            ff_store(ycur + c + 1 + u0 + j, dot);
          else
            sdotp[it] = dot;
        }
      }
      if (S > 1) {
        __syncthreads();
        for (int j = threadIdx.x; j < ncol; j += blockDim.x) {
          ff2 t = sdotp[j * S];
          for (int sg = 1; sg < S; ++sg) t = ff_add(t, sdotp[j * S + sg]);
          ff_store(ycur + c + 1 + u0 + j, t);
        }
      }
      __syncthreads();
      /* the block's share of y . x for the next step's alpha, in column order */
      ff2 dpart = ZERO;
      for (int j = threadIdx.x; j < ncol; j += blockDim.x) {
        const int r = c + 1 + u0 + j;
        dpart = ff_fma(ff_load(ycur + r), ff_load(svc + r), dpart);
      }
      const ff2 ds = ff_block_sum2(dpart, red);
      if (threadIdx.x == 0) ff_store(part_dot2 + (size_t)(c & 1) * G + b, ds);
    }
    TR_STAMP(c < early ? 2 : 1)
    target += G;
    if (!tr_grid_sync(count, target, err)) return false;
    TR_STAMP(4)
    tau_pf = tau_c;
    scale_pf = scale_cf;
    e_pf = beta;
    have_p = true;
  }
#undef TR_STAMP
  return true;
}

/* the last diagonal entry and the storage of the last reflector after the whole-matrix steps
 * (block 0) */
__device__ __forceinline__ void tr_full_last(double *A, int n, double *d, double *ybuf,
                                             double *part_dot2, ff2 tau_pf, ff2 e_pf,
                                             bool have_p)
{
  __shared__ ff2 s_slotf;
  const int G = gridDim.x, b = blockIdx.x;
  const ff2 ZERO = ff_make(0.f, 0.f);
  if (b == 0) {
    ff2 dsum = ZERO;
    if (have_p) dsum = ff_sum_partials(part_dot2 + (size_t)((n - 2) & 1) * G, G, &s_slotf);
    if (threadIdx.x == 0) {
      ff2 a = ff_load(A + (int64_t)(n - 1) * n + n - 1);
      if (have_p) {
        const ff2 alpha_p = ff_scale(ff_mul(ff_mul(tau_pf, tau_pf), dsum), -0.5f);
        const ff2 wp =
            ff_fma(tau_pf, ff_load(ybuf + (int64_t)((n - 2) & 1) * n + n - 1), alpha_p);
        a = ff_add(a, ff_neg(wp));
        a = ff_add(a, ff_neg(wp));
        A[(int64_t)(n - 2) * n + n - 1] = ff_to_double(e_pf);
      }
      d[n - 1] = ff_to_double(a);
    }
  }
}

__global__ void __launch_bounds__(TR_THREADS, 1)
k_tridiag(double *A, int n, double *d, double *e, double *tau, double *vbuf, double *wbuf,
          double *ybuf, double *part_dot2, unsigned *bar, int *err,
          unsigned long long *phase_ns)
{
  extern __shared__ double sh[];
  const ff2 ZERO = ff_make(0.f, 0.f);
  unsigned target = 0;
  ff2 tau_pf = ZERO, scale_pf = ZERO, e_pf = ZERO;
  bool have_p = false;
  /* phase_ns (optional, block 0): time in A, B (entry 1; entry 2 for the first 30% of the
   * steps) and the barrier (entry 4) */
  __shared__ unsigned long long s_ph[6];
  const bool stamp = phase_ns != NULL && blockIdx.x == 0 && threadIdx.x == 0;
  if (stamp) {
    for (int i = 0; i < 5; ++i) s_ph[i] = 0ull;
    s_ph[5] = globaltimer_ns();
  }
  if (!tr_full_steps(A, n, 0, d, e, tau, vbuf, wbuf, ybuf, part_dot2, bar, target, err, sh,
                     sh + n, sh + 2 * n, tau_pf, scale_pf, e_pf, have_p, NULL, 0, 0,
                     stamp ? s_ph : NULL))
    return;
  if (stamp)
    for (int i = 0; i < 5; ++i) phase_ns[i] = s_ph[i];
  tr_full_last(A, n, d, ybuf, part_dot2, tau_pf, e_pf, have_p);
}

/* ---------------------------------------------------------------------------------- */
/*
 * The same reduction (dsytd2, lower) with the trailing matrix held as its lower triangle only,
 * in TT x TT tiles: half the bytes per column step and two thirds of the float-float work of
 * the whole-column step, whose product needs both triangles.  Tile (I, J), I >= J, of the
 * lower triangle is TT*TT float-float pairs at Tm + tt_tile(I, J)*TT*TT, column-major inside
 * the tile (element (i, j) at j*TT + i); diagonal tiles are held in full; rows and columns
 * beyond n are zero padding.
 *
 * Work is split into parts: tile row I (TT rows) x column unit u (TT_U columns, u = 0 ..
 * nt*TT/TT_U - 1, in tile column u/(TT/TT_U)).  The blocks form a pr x pc grid: block (a, b)
 * owns the parts of the tile rows in row group a and the column units in column group b
 * (tables computed by the host for each first active tile index J0, balanced so that every
 * block has about the same number of parts).  So the product's index block K (TT indices)
 * has pc row-part contributors (blocks (rg(K), *)) and, for each of its units, pr column-part
 * contributors (blocks (*, cg(u))).  Per step:
 *   A   as in the whole-column step (every block: v and w of step c-1, the pending update of
 *       column c read from the tiles, its norm, the reflector; y.v from the index blocks'
 *       partial dots)
 *   B   each warp takes parts of the block: the pending rank-2 update of step c-1 (written
 *       back), the row dots (two rows per lane) and, off the diagonal, the column dots (a
 *       reduce-scatter over the warp per 4 columns); the block sums its parts per tile row and
 *       per column unit in a fixed order and publishes them, one arrival (release) on the
 *       index block's counter per published sum; block K mod G waits (acquire, bounded) for
 *       index block K's pc + (TT/TT_U)*pr arrivals and sums them in a fixed order into y and
 *       the index block's partial y.v
 *   --- grid barrier
 * Rows and columns up to c keep their values (the pending-update vectors and v are zero there),
 * so that phase A of a block still reading column c never sees it change.  Every sum has a
 * fixed order.
 */
#define TT 64
#define TT_U 16                /* columns per column unit */
#define TT_UPT (TT / TT_U)     /* column units per tile column */
#define TT_MAXG 32             /* row or column groups at most */
#define TR_ERR_LISTS 12
#define TR_ERR_WAIT 13

__host__ __device__ __forceinline__ int64_t tt_tile(int I, int J)
{
  return (int64_t)I * (I + 1) / 2 + J;
}

/* the lower triangle of the symmetric FP64 matrix A (column-major, both triangles valid) into
 * float-float tiles, padding zero */
__global__ void k_tri_to_tiles(const double *A, int n, int nt, double *Tm)
{
  const int64_t ntiles = (int64_t)nt * (nt + 1) / 2;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int I = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while ((int64_t)(I + 1) * (I + 2) / 2 <= t) ++I;
    while ((int64_t)I * (I + 1) / 2 > t) --I;
    const int J = (int)(t - (int64_t)I * (I + 1) / 2);
    double *tile = Tm + t * (TT * TT);
    for (int idx = threadIdx.x; idx < TT * TT; idx += blockDim.x) {
      const int j = idx / TT, i = idx - j * TT;
      const int r = I * TT + i, q = J * TT + j;
      const double v = (r < n && q < n) ? A[(int64_t)q * n + r] : 0.0;
      ff_store(tile + idx, ff_from_double(v));
    }
  }
}

/* a - (p q + r s) in float-float (the rank-2 update of one element): the two high products
 * exactly (TwoProd with FMA), their cross terms and the errors of two TwoSums gathered in one
 * FP32 term, one renormalisation: 27 FP32 operations against 30 for two ff_fma, of the same
 * error order.  With p = r = 0 or q = s = 0 it returns a normalised a unchanged. */
__device__ __forceinline__ ff2 ff_sub2prod(ff2 a, ff2 p, ff2 q, ff2 r, ff2 s)
{
  const float p1 = __fmul_rn(p.h, q.h);
  float e = __fmaf_rn(p.h, q.h, -p1);
  e = __fmaf_rn(p.h, q.l, e);
  e = __fmaf_rn(p.l, q.h, e);
  const float p2 = __fmul_rn(r.h, s.h);
  e = __fadd_rn(__fmaf_rn(r.h, s.h, -p2), e);
  e = __fmaf_rn(r.h, s.l, e);
  e = __fmaf_rn(r.l, s.h, e);
  const float t1 = __fsub_rn(a.h, p1);
  const float b1 = __fsub_rn(t1, a.h);
  const float r1 = __fadd_rn(__fsub_rn(a.h, __fsub_rn(t1, b1)), __fsub_rn(-p1, b1));
  const float t2 = __fsub_rn(t1, p2);
  const float b2 = __fsub_rn(t2, t1);
  const float r2 = __fadd_rn(__fsub_rn(t1, __fsub_rn(t2, b2)), __fsub_rn(-p2, b2));
  const float low = __fadd_rn(__fsub_rn(a.l, e), __fadd_rn(r1, r2));
  const float h = __fadd_rn(t2, low);
  return ff_make(h, __fsub_rn(low, __fsub_rn(h, t2)));
}

/* a x + b y in float-float: two exact high products, one TwoSum, the cross terms and errors
 * in one FP32 term (19 FP32 operations against 22 for ff_mul + ff_fma) */
__device__ __forceinline__ ff2 ff_dot2(ff2 a, ff2 x, ff2 b, ff2 y)
{
  const float p1 = __fmul_rn(a.h, x.h);
  float e = __fmaf_rn(a.h, x.h, -p1);
  e = __fmaf_rn(a.h, x.l, e);
  e = __fmaf_rn(a.l, x.h, e);
  const float p2 = __fmul_rn(b.h, y.h);
  e = __fadd_rn(__fmaf_rn(b.h, y.h, -p2), e);
  e = __fmaf_rn(b.h, y.l, e);
  e = __fmaf_rn(b.l, y.h, e);
  const float s = __fadd_rn(p1, p2);
  const float bb = __fsub_rn(s, p1);
  const float er = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, bb)), __fsub_rn(p2, bb));
  const float low = __fadd_rn(e, er);
  const float h = __fadd_rn(s, low);
  return ff_make(h, __fsub_rn(low, __fsub_rn(h, s)));
}

/* acc += a x with the accumulator left unnormalised (acc.h the running TwoSum of the high
 * products, acc.l every lower-order term): 12 FP32 operations against 15 for ff_fma; over a
 * short dot (16 terms here) its error stays of the order of the normalised accumulation's.
 * ff_renorm makes the pair normalised again. */
__device__ __forceinline__ ff2 ff_acc_lazy(ff2 acc, ff2 a, ff2 x)
{
  const float p = __fmul_rn(a.h, x.h);
  float e = __fmaf_rn(a.h, x.h, -p);
  e = __fmaf_rn(a.h, x.l, e);
  e = __fmaf_rn(a.l, x.h, e);
  const float s = __fadd_rn(acc.h, p);
  const float bb = __fsub_rn(s, acc.h);
  const float er = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  return ff_make(s, __fadd_rn(acc.l, __fadd_rn(e, er)));
}
__device__ __forceinline__ ff2 ff_renorm(ff2 a)
{
  const float h = __fadd_rn(a.h, a.l);
  return ff_make(h, __fsub_rn(a.l, __fsub_rn(h, a.h)));
}

/* one part (TT_U columns from TT*J + j0) of tile (I, J) by one warp: the pending update of
 * step c-1 (have_p), written back; the row dots with v over these columns into rs[TT] (rows
 * 2 lane, 2 lane + 1); unless the tile is diagonal, the column dots with v over the tile's
 * rows into cs[TT_U] */
__device__ __forceinline__ void tt_part(double *tile, int I, int J, int j0, bool diag,
                                        bool have_p, const double *svp, const double *swp,
                                        const double *svc, double *rs, double *cs, int lane)
{
  const ff2 ZERO = ff_make(0.f, 0.f);
  const int r = I * TT + 2 * lane;
  const ff2 vr0 = ff_load(svc + r), vr1 = ff_load(svc + r + 1);
  const ff2 pr0 = ff_load(svp + r), pr1 = ff_load(svp + r + 1);
  const ff2 qr0 = ff_load(swp + r), qr1 = ff_load(swp + r + 1);
  ff2 ra0 = ZERO, ra1 = ZERO;
  const int col0 = J * TT + j0;
  double *p0 = tile + (size_t)j0 * TT + 2 * lane;
#pragma unroll 1
  for (int cb = 0; cb < TT_U; cb += 4) {
    float4 a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = *reinterpret_cast<const float4 *>(p0 + (size_t)(cb + k) * TT);
    ff2 cp[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int col = col0 + cb + k;
      ff2 a0 = ff_make(a[k].x, a[k].y), a1 = ff_make(a[k].z, a[k].w);
      if (have_p) {
        const ff2 vpc = ff_load(svp + col), wpc = ff_load(swp + col);
        a0 = ff_sub2prod(a0, pr0, wpc, qr0, vpc);
        a1 = ff_sub2prod(a1, pr1, wpc, qr1, vpc);
        *reinterpret_cast<float4 *>(p0 + (size_t)(cb + k) * TT) = make_float4(a0.h, a0.l, a1.h, a1.l);
      }
      const ff2 vc = ff_load(svc + col);
      ra0 = ff_acc_lazy(ra0, a0, vc);
      ra1 = ff_acc_lazy(ra1, a1, vc);
      cp[k] = ff_dot2(a0, vr0, a1, vr1);
    }
    if (!diag) {
      /* reduce-scatter over the warp: lanes 8t..8t+7 end with column cb + t (lane bits 4 and 3
       * pick the column, bits 2..0 are summed) */
      const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const ff2 send = b4 ? cp[k] : cp[k + 2];
        const ff2 keep = b4 ? cp[k + 2] : cp[k];
        cp[k] = ff_add(keep, ff_shfl_xor(send, 16));
      }
      {
        const ff2 send = b3 ? cp[0] : cp[1];
        const ff2 keep = b3 ? cp[1] : cp[0];
        cp[0] = ff_add(keep, ff_shfl_xor(send, 8));
      }
      cp[0] = ff_add(cp[0], ff_shfl_xor(cp[0], 4));
      cp[0] = ff_add(cp[0], ff_shfl_xor(cp[0], 2));
      cp[0] = ff_add(cp[0], ff_shfl_xor(cp[0], 1));
      if ((lane & 7) == 0) ff_store(cs + cb + (lane >> 3), cp[0]);
    }
  }
  ff_store(rs + 2 * lane, ff_renorm(ra0));
  ff_store(rs + 2 * lane + 1, ff_renorm(ra1));
}

/* shared-memory bytes of k_tridiag_tiled for round size R (parts per round) and the bounds of
 * a block's tile rows, column units and parts */
__host__ __device__ inline size_t tt_smem_bytes(int nt, int R, int maxr, int maxc, int maxi)
{
  const size_t npad = (size_t)nt * TT;
  const size_t dbl = 3 * npad + (size_t)R * (TT + TT_U) + (size_t)maxr * TT + (size_t)maxc * TT_U;
  const size_t bytes = dbl * sizeof(double) + (size_t)maxi * sizeof(int4) +
                       sizeof(int) * (size_t)(3 * maxr + maxc) + (size_t)nt * (1 + TT_UPT);
  return (bytes + 15) & ~(size_t)15;
}

/*
 * Tm: the tiles (k_tri_to_tiles); A receives the reflectors in FP64 in A(c+2:n, c) and e on the
 * subdiagonal, as dormtr (lower) reads them.  rgt [nt][nt], cgt [nt][nt*TT_UPT]: the row group
 * of each tile row and the column group of each column unit for first active tile index J0
 * (row J0 of each table).  prow [nt][pc][TT], pcol [nt*TT_UPT][pr][TT_U]: the published row
 * and column parts; dotp [2][nt]: the index blocks' partial y.v of alternate steps; kcnt [nt]:
 * arrival counters (zero at launch).  maxr/maxc/maxi bound a block's tile rows, column units
 * and parts over all J0; R parts per round.  Steps from cs on run whole columns
 * (tr_full_steps), part_dot2 [2G] their block partials.
 */
__global__ void __launch_bounds__(TR_THREADS, 1)
k_tridiag_tiled(double *A, double *Tm, int n, int nt, int pr, int pc, int maxr, int maxc,
                int maxi, int R, int cs, const unsigned char *rgt, const unsigned char *cgt,
                double *d, double *e, double *tau, double *vbuf, double *wbuf, double *ybuf,
                double *prow, double *pcol, double *dotp, unsigned *kcnt, double *part_dot2,
                unsigned *bar, int *err, unsigned long long *phase_ns)
{
  extern __shared__ double sh[];
  const int npad = nt * TT, nu = nt * TT_UPT;
  double *svp = sh, *swp = sh + npad, *svc = sh + 2 * npad; /* float-float pairs */
  double *rslot = sh + 3 * (size_t)npad;      /* [R][TT] */
  double *cslot = rslot + (size_t)R * TT;     /* [R][TT_U] */
  double *racc = cslot + (size_t)R * TT_U;    /* [maxr][TT] */
  double *cacc = racc + (size_t)maxr * TT;    /* [maxc][TT_U] */
  int4 *items = reinterpret_cast<int4 *>(cacc + (size_t)maxc * TT_U);
  int *rowl = reinterpret_cast<int *>(items + maxi); /* tile rows */
  int *rowb = rowl + maxr;                           /* first part of each tile row */
  int *rown = rowb + maxr;                           /* parts of each tile row */
  int *coll = rown + maxr;                           /* column units */
  unsigned char *rg = reinterpret_cast<unsigned char *>(coll + maxc);
  unsigned char *cg = rg + nt;
  __shared__ ff2 red[TR_WARPS];
  __shared__ ff2 s_dot[TR_WARPS];
  __shared__ tr_step st;
  __shared__ ff2 s_slotf, s_dc;
  __shared__ int s_nr, s_nc, s_ni, s_ok;
  const int G = gridDim.x, b = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool active = b < pr * pc;
  const int ga = active ? b / pc : 0, gb = active ? b - (b / pc) * pc : 0;
  const ff2 ONE = ff_make(1.f, 0.f), ZERO = ff_make(0.f, 0.f);
  unsigned *count = bar;
  unsigned target = 0;
  /* the previous step's reflector scalars (block-uniform, kept in shared memory) */
  __shared__ ff2 s_tau_p, s_scale_p, s_e_p;
  bool have_p = false;
  /* phase_ns (optional, block 0): time in A, B (entry 1; entry 2 for the first 30% of the
   * steps) and the barrier (entry 4), accumulated in shared memory */
  __shared__ unsigned long long s_ph[6];
  const bool stamp = phase_ns != NULL && b == 0 && threadIdx.x == 0;
  if (stamp) {
    for (int i = 0; i < 5; ++i) s_ph[i] = 0ull;
    s_ph[5] = globaltimer_ns();
  }
  if (threadIdx.x == 0) s_tau_p = s_scale_p = s_e_p = ZERO;
#define TT_STAMP(i)                                    \
  if (stamp) {                                         \
    const unsigned long long t_now = globaltimer_ns(); \
    s_ph[i] += t_now - s_ph[5];                        \
    s_ph[5] = t_now;                                   \
  }
  const int early = (int)((3LL * n) / 10);
  const unsigned arrivals = (unsigned)(pc + TT_UPT * pr); /* per index block and step */
  for (int q = threadIdx.x; q < 3 * npad; q += blockDim.x) sh[q] = 0.0; /* padding stays 0 */
  int j0_lists = -1;
  for (int c = 0; c < cs; ++c) {
    const int J0 = (c + 1) / TT;
    if (J0 != j0_lists) {
      /* the block's tile rows, column units and parts from J0 on (row J0 of the tables) */
      for (int I = threadIdx.x; I < nt; I += blockDim.x) rg[I] = rgt[(size_t)J0 * nt + I];
      for (int u = threadIdx.x; u < nu; u += blockDim.x) cg[u] = cgt[(size_t)J0 * nu + u];
      __syncthreads();
      if (threadIdx.x == 0) {
        int nr = 0, nc = 0, ni = 0, bad = 0;
        if (active) {
          for (int I = J0; I < nt; ++I)
            if (rg[I] == ga) {
              if (nr < maxr) rowl[nr++] = I; else bad = 1;
            }
          for (int u = J0 * TT_UPT; u < nu; ++u)
            if (cg[u] == gb) {
              if (nc < maxc) coll[nc++] = u; else bad = 1;
            }
          for (int kr = 0; kr < nr; ++kr) {
            rowb[kr] = ni;
            int k = 0;
            for (; k < nc && coll[k] / TT_UPT <= rowl[kr]; ++k) {
              if (ni < maxi)
                items[ni++] = make_int4(rowl[kr], coll[k], kr,
                                        coll[k] / TT_UPT == rowl[kr] ? -1 : k);
              else
                bad = 1;
            }
            rown[kr] = k;
          }
        }
        if (bad) atomicExch(err, TR_ERR_LISTS);
        s_nr = nr;
        s_nc = nc;
        s_ni = ni;
      }
      __syncthreads();
      j0_lists = J0;
    }
    /* ---- A: as in the whole-column step, with column c read from the tiles ---- */
    const ff2 tau_pf = s_tau_p, scale_pf = s_scale_p, e_pf = s_e_p;
    double *xcur = (c & 1) ? wbuf : vbuf, *xprev = (c & 1) ? vbuf : wbuf;
    double *ycur = ybuf + (int64_t)(c & 1) * n, *yprev = ybuf + (int64_t)((c + 1) & 1) * n;
    ff2 pacc = ZERO;
    if (have_p && warp == TR_WARPS - 1) {
      /* y.v of step c-1: its index blocks' partial dots (from (c-1+1)/TT on), in order */
      const double *pprev = dotp + (size_t)((c + 1) & 1) * nt;
      for (int k = c / TT + lane; k < nt; k += 32) pacc = ff_add(pacc, ff_load(pprev + k));
    }
    {
      const int Jc = c / TT, jc = c - Jc * TT;
#pragma unroll 4
      for (int q = c + threadIdx.x; q < n; q += blockDim.x) {
        ff2 vp = ZERO, yq = ZERO;
        if (have_p) {
          vp = (q == c) ? ONE : ff_mul(ff_load(xprev + q), scale_pf);
          yq = ff_load(yprev + q);
        }
        ff_store(svp + q, vp);
        ff_store(swp + q, yq);
        const int I = q / TT;
        ff_store(svc + q, ff_load(Tm + (tt_tile(I, Jc) * TT + jc) * TT + (q - I * TT)));
      }
    }
    if (have_p && warp == TR_WARPS - 1) {
      for (int o = 16; o; o >>= 1) pacc = ff_add(pacc, ff_shfl_xor(pacc, o));
      if (lane == 0) s_slotf = pacc;
    }
    __syncthreads();
    ff2 wpc = ZERO, alpha_pf = ZERO;
    if (have_p) {
      const ff2 dsum = s_slotf;
      alpha_pf = ff_scale(ff_mul(ff_mul(tau_pf, tau_pf), dsum), -0.5f);
      wpc = ff_fma(tau_pf, ff_load(swp + c), alpha_pf);
    }
    {
      const int cnt = n - c, per = (cnt + G - 1) / G;
      const int r0 = c + b * per, r1 = min(n, r0 + per);
      ff2 nrm = ZERO;
      for (int q = c + threadIdx.x; q < n; q += blockDim.x) {
        ff2 x = ff_load(svc + q);
        const bool mine = q >= r0 && q < r1;
        if (have_p) {
          const ff2 vp = ff_load(svp + q);
          const ff2 wp = ff_fma(tau_pf, ff_load(swp + q), ff_mul(alpha_pf, vp));
          ff_store(swp + q, wp);
          x = ff_fma(ff_neg(vp), wpc, x);
          x = ff_add(x, ff_neg(wp));
          if (mine) A[(int64_t)(c - 1) * n + q] = ff_to_double(q == c ? e_pf : vp);
        }
        ff_store(svc + q, x);
        if (mine) ff_store(xcur + q, x);
        if (q >= c + 2) nrm = ff_fma(x, x, nrm);
      }
      const ff2 xn2 = ff_block_sum2(nrm, red);
      if (threadIdx.x == 0) {
        const ff2 alpha = ff_load(svc + c + 1);
        s_dc = ff_load(svc + c);
        if (xn2.h == 0.f) {
          st.beta = alpha;
          st.tau_c = ZERO;
          st.scale_c = ZERO;
        } else {
          const ff2 nrm2 = ff_sqrt(ff_fma(alpha, alpha, xn2));
          const ff2 beta = alpha.h >= 0.f ? ff_neg(nrm2) : nrm2;
          const ff2 am = ff_add(alpha, ff_neg(beta));
          st.beta = beta;
          st.tau_c = ff_div(ff_neg(am), beta);
          st.scale_c = ff_div(ONE, am);
        }
      }
      __syncthreads();
      if (b == 0 && threadIdx.x == 32) {
        d[c] = ff_to_double(s_dc);
        e[c] = ff_to_double(st.beta);
        tau[c] = ff_to_double(st.tau_c);
      }
    }
    const ff2 beta = st.beta, tau_c = st.tau_c;
    const ff2 scale_cf = st.scale_c;
    TT_STAMP(0)
    /* ---- B ---- v of step c; the vectors zero at indices J0*TT .. c (rows and columns up to
     * c keep their values, and take no part in the dots) */
    for (int q = c + 1 + threadIdx.x; q < n; q += blockDim.x)
      ff_store(svc + q, (q == c + 1) ? ONE : ff_mul(ff_load(svc + q), scale_cf));
    for (int q = J0 * TT + threadIdx.x; q <= c; q += blockDim.x) {
      ff_store(svc + q, ZERO);
      ff_store(svp + q, ZERO);
      ff_store(swp + q, ZERO);
    }
    const int nr = s_nr, nc = s_nc, ni = s_ni;
    for (int idx = threadIdx.x; idx < nr * TT + nc * TT_U; idx += blockDim.x)
      ff_store(idx < nr * TT ? racc + idx : cacc + (idx - nr * TT), ZERO);
    __syncthreads();
    for (int rb = 0; rb < ni; rb += R) {
      const int re = min(ni, rb + R);
      for (int u = warp; rb + u < re; u += TR_WARPS) {
        const int4 it = items[rb + u];
        const int I = it.x, J = it.y / TT_UPT, j0 = (it.y - J * TT_UPT) * TT_U;
        double *rs = rslot + (size_t)u * TT, *cs_ = cslot + (size_t)u * TT_U;
        if (J == J0 && J0 * TT + j0 + TT_U <= c + 1) {
          /* every column of this part is at or before c */
          ff_store(rs + 2 * lane, ZERO);
          ff_store(rs + 2 * lane + 1, ZERO);
          if (lane < TT_U) ff_store(cs_ + lane, ZERO);
        } else {
          tt_part(Tm + tt_tile(I, J) * (TT * TT), I, J, j0, I == J, have_p, svp, swp, svc, rs,
                  cs_, lane);
        }
      }
      __syncthreads();
      /* the round's parts into the block's sums, in part order: tile row kr owns parts
       * rowb[kr] .. rowb[kr] + rown[kr] - 1, its k-th column unit at rowb[kr] + k */
      for (int idx = threadIdx.x; idx < nr * TT; idx += blockDim.x) {
        const int kr = idx / TT, i = idx - kr * TT;
        ff2 s = ff_load(racc + idx);
        const int t0 = max(rb, rowb[kr]), t1 = min(re, rowb[kr] + rown[kr]);
        for (int t = t0; t < t1; ++t) s = ff_add(s, ff_load(rslot + (size_t)(t - rb) * TT + i));
        ff_store(racc + idx, s);
      }
      for (int idx = threadIdx.x; idx < nc * TT_U; idx += blockDim.x) {
        const int kc = idx / TT_U, j = idx - kc * TT_U;
        ff2 s = ff_load(cacc + idx);
        for (int kr = 0; kr < nr; ++kr) {
          const int t = rowb[kr] + kc;
          if (kc < rown[kr] && coll[kc] / TT_UPT != rowl[kr] && t >= rb && t < re)
            s = ff_add(s, ff_load(cslot + (size_t)(t - rb) * TT_U + j));
        }
        ff_store(cacc + idx, s);
      }
      __syncthreads();
    }
    /* publish the block's sums: row parts of its tile rows, column parts of its units; then
     * one arrival per published sum on its index block's counter */
    if (active) {
      for (int idx = threadIdx.x; idx < nr * TT; idx += blockDim.x) {
        const int kr = idx / TT, i = idx - kr * TT;
        ff_store(prow + ((size_t)rowl[kr] * pc + gb) * TT + i, ff_load(racc + idx));
      }
      for (int idx = threadIdx.x; idx < nc * TT_U; idx += blockDim.x) {
        const int kc = idx / TT_U, j = idx - kc * TT_U;
        ff_store(pcol + ((size_t)coll[kc] * pr + ga) * TT_U + j, ff_load(cacc + idx));
      }
    }
    __syncthreads();
    if (active) {
      if ((int)threadIdx.x < nr) /* nr, nc <= 512 (host check) */
        red_release_gpu(kcnt + rowl[threadIdx.x], 1u);
      else if (threadIdx.x >= 512 && (int)threadIdx.x - 512 < nc)
        red_release_gpu(kcnt + coll[threadIdx.x - 512] / TT_UPT, 1u);
    }
    /* index blocks K = b, b + G, ...: wait for their arrivals, then y over the TT indices
     * (pc row parts, then pr column parts of the index's unit, in order: 16 threads per index
     * with two terms each and a fixed shuffle tree) and the partial y.v */
    {
      const unsigned ktarget = arrivals * (unsigned)(c + 1);
      for (int K = b; K < nt; K += G) {
        if (K < J0) continue;
        if (threadIdx.x == 0) {
          int ok = 1;
          volatile int *verr = err;
          const uint64_t t0 = globaltimer_ns();
          for (unsigned it = 1; ld_acquire_gpu(kcnt + K) < ktarget; ++it) {
            if ((it & 63u) == 0) {
              if (*verr) {
                ok = 0;
                break;
              }
              if (globaltimer_ns() - t0 > GP_WAIT_NS) {
                atomicExch(err, TR_ERR_WAIT);
                ok = 0;
                break;
              }
            }
          }
          s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) return;
        const int i = threadIdx.x >> 4, g = threadIdx.x & 15;
        const int nterm = pc + pr;
        ff2 y = ZERO;
        for (int t = g; t < nterm; t += 16) {
          const double *src = t < pc ? prow + ((size_t)K * pc + t) * TT + i
                                     : pcol + ((size_t)(K * TT_UPT + i / TT_U) * pr + (t - pc)) *
                                                  TT_U + (i & (TT_U - 1));
          y = ff_add(y, ff_load(src));
        }
        for (int o = 8; o; o >>= 1) y = ff_add(y, ff_shfl_xor(y, o));
        const int q = K * TT + i;
        ff2 dv = ZERO;
        if (g == 0) {
          if (q < n) ff_store(ycur + q, y);
          dv = ff_mul(y, ff_load(svc + q));
        }
        dv = ff_add(dv, ff_shfl_xor(dv, 16)); /* the warp's two indices, lanes 0 and 16 */
        if (lane == 0) s_dot[warp] = dv;
        __syncthreads();
        if (threadIdx.x < 32) {
          ff2 t = s_dot[threadIdx.x];
          for (int o = 16; o; o >>= 1) t = ff_add(t, ff_shfl_xor(t, o));
          if (threadIdx.x == 0) ff_store(dotp + (size_t)(c & 1) * nt + K, t);
        }
        __syncthreads();
      }
    }
    TT_STAMP(c < early ? 2 : 1)
    if (threadIdx.x == 0) { /* read again only after the grid barrier's block barriers */
      s_tau_p = tau_c;
      s_scale_p = scale_cf;
      s_e_p = beta;
    }
    target += G;
    if (!tr_grid_sync(count, target, err)) return;
    TT_STAMP(4)
    have_p = true;
  }
  if (cs < n - 1) {
    /* the switch to whole columns: the trailing block (indices >= cs) of the block's parts
     * into A as float-float pairs, both triangles (the pending update of step cs-1 is applied
     * by the first whole-column step) */
    const int ni = s_ni;
    for (int64_t idx = threadIdx.x; idx < (int64_t)ni * (TT * TT_U); idx += blockDim.x) {
      const int u = (int)(idx / (TT * TT_U)), rem = (int)(idx - (int64_t)u * (TT * TT_U));
      const int j = rem / TT, i = rem - j * TT;
      const int4 it = items[u];
      const int J = it.y / TT_UPT, jt = (it.y - J * TT_UPT) * TT_U + j;
      const int r = it.x * TT + i, q = J * TT + jt;
      if (r >= cs && q >= cs && r < n && q < n) {
        const double v = Tm[(tt_tile(it.x, J) * TT + jt) * TT + i];
        A[(int64_t)q * n + r] = v;
        if (it.x != J) A[(int64_t)r * n + q] = v;
      }
    }
    target += G;
    if (!tr_grid_sync(count, target, err)) return;
    ff2 tau_pf = s_tau_p, scale_pf = s_scale_p, e_pf = s_e_p;
    if (!tr_full_steps(A, n, cs, d, e, tau, vbuf, wbuf, ybuf, part_dot2, count, target, err, svp,
                       swp, svc, tau_pf, scale_pf, e_pf, have_p,
                       dotp + (size_t)((cs + 1) & 1) * nt, cs / TT, nt, stamp ? s_ph : NULL))
      return;
    if (stamp)
      for (int i = 0; i < 5; ++i) phase_ns[i] = s_ph[i];
    tr_full_last(A, n, d, ybuf, part_dot2, tau_pf, e_pf, have_p);
    return;
  }
  if (stamp)
    for (int i = 0; i < 5; ++i) phase_ns[i] = s_ph[i];
#undef TT_STAMP
  /* last diagonal entry and the storage of the last reflector */
  if (b == 0) {
    ff2 dsum = ZERO;
    if (have_p) {
      if (threadIdx.x < 32) {
        ff2 s = ZERO;
        const double *pl = dotp + (size_t)((n - 2) & 1) * nt;
        for (int k = (n - 1) / TT + (int)threadIdx.x; k < nt; k += 32) s = ff_add(s, ff_load(pl + k));
        for (int o = 16; o; o >>= 1) s = ff_add(s, ff_shfl_xor(s, o));
        if (threadIdx.x == 0) s_slotf = s;
      }
      __syncthreads();
      dsum = s_slotf;
    }
    if (threadIdx.x == 0) {
      const int Il = (n - 1) / TT, il = n - 1 - Il * TT;
      ff2 a = ff_load(Tm + (tt_tile(Il, Il) * TT + il) * TT + il);
      const ff2 tau_pf = s_tau_p, e_pf = s_e_p;
      if (have_p) {
        const ff2 alpha_p = ff_scale(ff_mul(ff_mul(tau_pf, tau_pf), dsum), -0.5f);
        const ff2 wp =
            ff_fma(tau_pf, ff_load(ybuf + (int64_t)((n - 2) & 1) * n + n - 1), alpha_p);
        a = ff_add(a, ff_neg(wp));
        a = ff_add(a, ff_neg(wp));
        A[(int64_t)(n - 2) * n + n - 1] = ff_to_double(e_pf);
      }
      d[n - 1] = ff_to_double(a);
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

/* block sum (fixed order: warp shuffles, then warp 0 over the warps' sums), broadcast to
 * every thread; red holds at least one double per warp */
__device__ double block_sum(double v, double *red)
{
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    double t = (int)threadIdx.x < nw ? red[threadIdx.x] : 0.0;
    for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
    if (threadIdx.x == 0) red[32] = t;
  }
  __syncthreads();
  const double r = red[32];
  __syncthreads();
  return r;
}

/*
 * Inverse iteration, one block per top eigenvalue (vector j belongs to w[n-1-j]).
 * The LU factorisation with partial pivoting of T - lam I and the solves are sequential
 * recurrences run by thread 0 with the running values carried in registers (the arrays are
 * only written, or read ahead of the dependency chain); the other threads normalise.
 * With in_smem, the factors, the iterate and (during the factorisation) d and e sit in shared
 * memory, 41 n bytes, so that the recurrences wait on shared-memory rather than L2 latency:
 * d is staged where the iterate goes later and e where the second superdiagonal of U is
 * written, each e(i) being read before DU2(i) overwrites it.  Otherwise work holds the
 * factors (per vector 6n doubles) and the iterate stays in Z.
 * Z [nvec][n] (column-major N x nvec).
 */
__global__ void k_inverse_iteration(const double *__restrict__ d, const double *__restrict__ e,
                                    int n, const double *__restrict__ w, int nvec, double tnorm,
                                    double *Z, double *work, int in_smem)
{
  __shared__ double red[256];
  extern __shared__ double ii_sm[];
  const int j = blockIdx.x;
  if (j >= nvec) return;
  double *base = in_smem ? ii_sm : work + (int64_t)j * 6 * n;
  double *Dinv = base, *DL = base + n, *DU = base + 2 * n, *DU2 = base + 3 * n;
  double *xg = Z + (int64_t)j * n;
  double *x = in_smem ? base + 4 * n : xg;
  uint8_t *piv = (uint8_t *)(base + 5 * n);
  const double *dd = d, *ee = e;
  if (in_smem) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      x[i] = d[i];
      if (i < n - 1) DU2[i] = e[i];
    }
    __syncthreads();
    dd = x;
    ee = DU2;
  }
  const double lam = w[n - 1 - j];
  const double tiny = DBL_EPSILON * tnorm;
  if (threadIdx.x == 0) {
    /* dgttrf-style elimination; cur = running diagonal of row i, du = its superdiagonal */
    double cur = dd[0] - lam;
    double du = n > 1 ? ee[0] : 0.0;
    for (int i = 0; i < n - 1; ++i) {
      const double ei = ee[i];
      const double dn = dd[i + 1] - lam;               /* row i+1 diagonal */
      const double en = (i < n - 2) ? ee[i + 1] : 0.0; /* row i+1 superdiagonal */
      /* one division per step: the pivot's reciprocal, then the multiplier from it */
      if (fabs(cur) >= fabs(ei)) {
        if (cur == 0.0) cur = tiny;
        const double rc = 1.0 / cur;
        double f = ei * rc;
        DL[i] = f;
        DU[i] = du;
        DU2[i] = 0.0;
        Dinv[i] = rc;
        piv[i] = 0;
        cur = dn - f * du;
        du = en;
      } else {
        const double re = 1.0 / ei;
        double f = cur * re;
        DL[i] = f;
        Dinv[i] = re;
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
  __syncthreads();
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
  for (int i = threadIdx.x; i < n; i += blockDim.x) xg[i] = x[i] * inv;
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

/*
 * Back-transformation Z := Q Z of the nvec eigenvectors of T (dormtr, side L, lower, no
 * transpose), Q = H(0) H(1) ... H(n-2) with H(i) = I - tau_i v_i v_i^T, v_i(i+1) = 1 and
 * v_i(i+2:n) stored in A(i+2:n, i).  The reflectors are taken WY_B at a time in the compact
 * WY form H(i0)...H(i0+b-1) = I - V T V^T (T upper triangular, LAPACK dlarft's forward
 * recurrence T(j,j) = tau_j, T(0:j,j) = -tau_j T(0:j,0:j) V(:,0:j)^T v_j), last block first,
 * Z := Z - V (T (V^T Z)).  T depends on the reflectors only, so k_wy_tmat builds every
 * block's T at once (one CTA per block) before k_apply_q runs the blocks in order.
 * Float-float arithmetic (about 46 bits) from the FP64 inputs to the FP64 output.
 */
#define WY_B 32
#define WY_THREADS 512
#define WT_THREADS 256
#define WT_ROWS 64

/* entry e of the upper triangle (row-major, k <= c) of a WY_B x WY_B matrix */
__device__ __forceinline__ void wy_upper_entry(int e, int *k, int *c)
{
  int r = 0;
  while (e >= WY_B - r) {
    e -= WY_B - r;
    ++r;
  }
  *k = r;
  *c = r + e;
}

/* Tg [nblk][WY_B][WY_B] (float-float pairs in doubles' storage): block blk's T, from
 * S = V^T V summed over the reflector rows in order (rows staged WT_ROWS at a time) */
__global__ void __launch_bounds__(WT_THREADS)
k_wy_tmat(const double *__restrict__ A, int n, const double *__restrict__ tau, double *Tg)
{
  __shared__ ff2 Vc[WT_ROWS][WY_B + 1];
  __shared__ ff2 Ss[WY_B][WY_B + 1];
  __shared__ ff2 Tm[WY_B][WY_B + 1];
  constexpr int NUP = WY_B * (WY_B + 1) / 2;
  constexpr int SLOTS = (NUP + WT_THREADS - 1) / WT_THREADS;
  const int blk = blockIdx.x, tid = threadIdx.x;
  const int nref = n - 1, i0 = blk * WY_B;
  if (i0 >= nref) return;
  const int nb = nref - i0 < WY_B ? nref - i0 : WY_B;
  const ff2 ZERO = ff_make(0.f, 0.f);
  int ek[SLOTS], ec[SLOTS];
  ff2 acc[SLOTS];
#pragma unroll
  for (int sl = 0; sl < SLOTS; ++sl) {
    const int e = tid + sl * WT_THREADS;
    ek[sl] = ec[sl] = -1;
    if (e < NUP) wy_upper_entry(e, &ek[sl], &ec[sl]);
    acc[sl] = ZERO;
  }
  for (int r0 = i0 + 1; r0 < n; r0 += WT_ROWS) {
    const int nr = n - r0 < WT_ROWS ? n - r0 : WT_ROWS;
    __syncthreads();
    for (int idx = tid; idx < WT_ROWS * WY_B; idx += WT_THREADS) {
      const int k = idx / WT_ROWS, q = idx - k * WT_ROWS, rr = r0 + q, i = i0 + k;
      double v = 0.0;
      if (k < nb && q < nr) v = rr == i + 1 ? 1.0 : (rr > i + 1 ? A[(size_t)i * n + rr] : 0.0);
      Vc[q][k] = ff_from_double(v);
    }
    __syncthreads();
#pragma unroll
    for (int sl = 0; sl < SLOTS; ++sl) {
      if (ek[sl] < 0) continue;
      ff2 t = acc[sl];
      for (int q = 0; q < nr; ++q) t = ff_fma(Vc[q][ek[sl]], Vc[q][ec[sl]], t);
      acc[sl] = t;
    }
  }
#pragma unroll
  for (int sl = 0; sl < SLOTS; ++sl)
    if (ek[sl] >= 0) Ss[ek[sl]][ec[sl]] = acc[sl];
  __syncthreads();
  /* T (dlarft forward, columnwise): one warp, column j after column j-1 */
  if (tid < 32) {
    for (int j = 0; j < WY_B; ++j) {
      const ff2 tj = j < nb ? ff_from_double(tau[i0 + j]) : ZERO;
      ff2 t = ZERO;
      if (tid < j) t = ff_neg(ff_mul(tj, Ss[tid][j]));
      /* T(0:j, j) = T(0:j, 0:j) t: row tid of the upper triangle */
      ff2 a = ZERO;
      for (int l = 0; l < j; ++l) {
        const ff2 tl = ff_make(__shfl_sync(0xFFFFFFFFu, t.h, l), __shfl_sync(0xFFFFFFFFu, t.l, l));
        if (tid <= l) a = ff_fma(Tm[tid][l], tl, a);
      }
      if (tid < j) Tm[tid][j] = a;
      if (tid == j) Tm[j][j] = tj;
      if (tid > j) Tm[tid][j] = ZERO;
      __syncwarp();
    }
  }
  __syncthreads();
  double *T = Tg + (size_t)blk * WY_B * WY_B;
  for (int idx = tid; idx < WY_B * WY_B; idx += WT_THREADS)
    ff_store(T + idx, Tm[idx / WY_B][idx % WY_B]);
}

/*
 * One cooperative launch, one CTA per SM with a fixed slab of rows: per block of reflectors
 * each CTA forms its rows' share of V^T Z (partials), a grid barrier, the partials are summed
 * in fixed order (entries spread over the CTAs), a second barrier, then every CTA forms
 * W = T (V^T Z) with the block's T from k_wy_tmat and updates its own rows.  Bounded grid
 * barriers report through err.
 */
__global__ void __launch_bounds__(WY_THREADS, 1)
k_apply_q(const double *__restrict__ A, int n, const double *__restrict__ Tg, double *Z, int nvec,
          double *part, double *S, unsigned *bar, int *err)
{
  /* all products in float-float on the FP32 pipe (GB300's FP64 pipe issues ~2 FMAs per
   * clock per SM); part and S hold float-float pairs in doubles' storage */
  extern __shared__ double wsm[];
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int rpb = (n + G - 1) / G;
  const int R0 = b * rpb < n ? b * rpb : n, R1 = R0 + rpb < n ? R0 + rpb : n;
  const int nent = WY_B * nvec;
  ff2 *Vs = reinterpret_cast<ff2 *>(wsm);    /* [rpb][WY_B]  the CTA's rows of V */
  ff2 *Zs = Vs + (size_t)rpb * WY_B;         /* [rpb][nvec]  its rows of Z */
  ff2 *Ss = Zs + (size_t)rpb * nvec;         /* [WY_B][nvec] V^T Z */
  ff2 *Tm = Ss + (size_t)nent;               /* [WY_B][WY_B] */
  ff2 *Wm = Tm + WY_B * WY_B;                /* [WY_B][nvec] */
  const ff2 ZERO = ff_make(0.f, 0.f);
  unsigned target = 0;
  const int nr = R1 - R0;
  for (int idx = tid; idx < nr * nvec; idx += WY_THREADS) {
    const int c = idx / nr, r = idx - c * nr;
    Zs[r * nvec + c] = ff_from_double(Z[(size_t)c * n + R0 + r]);
  }
  const int nref = n - 1;
  const int nblk = (nref + WY_B - 1) / WY_B;
  for (int blk = nblk - 1; blk >= 0; --blk) {
    const int i0 = blk * WY_B, nb = nref - i0 < WY_B ? nref - i0 : WY_B;
    const int r0 = R0 > i0 + 1 ? R0 : i0 + 1;  /* V is zero above row i0+1 */
    const int m = r0 < R1 ? R1 - r0 : 0;
    __syncthreads();
    for (int idx = tid; idx < m * WY_B; idx += WY_THREADS) {
      const int k = idx / m, rr = r0 + (idx - k * m);
      const int i = i0 + k;
      double v = 0.0;
      if (k < nb) v = rr == i + 1 ? 1.0 : (rr > i + 1 ? A[(size_t)i * n + rr] : 0.0);
      Vs[(rr - R0) * WY_B + k] = ff_from_double(v);
    }
    __syncthreads();
    /* partial V^T Z over the CTA's rows */
    for (int e = tid; e < nent; e += WY_THREADS) {
      const int k = e / nvec, c = e - k * nvec;
      ff2 acc = ZERO;
      for (int rr = r0 - R0; rr < R1 - R0; ++rr)
        acc = ff_fma(Vs[rr * WY_B + k], Zs[rr * nvec + c], acc);
      ff_store(part + (size_t)b * nent + e, acc);
    }
    target += G;
    if (!tr_grid_sync(bar, target, err)) return;
    /* one warp per entry: lanes sum every 32nd partial, then a fixed shuffle tree */
    {
      const int lane = tid & 31, gw = b * (WY_THREADS / 32) + (tid >> 5);
      for (int e = gw; e < nent; e += G * (WY_THREADS / 32)) {
        ff2 acc = ZERO;
        for (int g = lane; g < G; g += 32) acc = ff_add(acc, ff_load(part + (size_t)g * nent + e));
        for (int o = 16; o; o >>= 1) acc = ff_add(acc, ff_shfl_xor(acc, o));
        if (lane == 0) ff_store(S + e, acc);
      }
    }
    target += G;
    if (!tr_grid_sync(bar, target, err)) return;
    if (m == 0) continue;
    for (int e = tid; e < nent; e += WY_THREADS) Ss[e] = ff_load(S + e);
    for (int e = tid; e < WY_B * WY_B; e += WY_THREADS)
      Tm[e] = ff_load(Tg + (size_t)blk * WY_B * WY_B + e);
    __syncthreads();
    /* W = T (V^T Z) */
    for (int e = tid; e < WY_B * nvec; e += WY_THREADS) {
      const int k = e / nvec, c = e - k * nvec;
      ff2 acc = ZERO;
      for (int l = k; l < WY_B; ++l) acc = ff_fma(Tm[k * WY_B + l], Ss[l * nvec + c], acc);
      Wm[e] = acc;
    }
    __syncthreads();
    /* Z(rows) -= V(rows) W */
    for (int idx = tid; idx < m * nvec; idx += WY_THREADS) {
      const int rr = (r0 - R0) + idx / nvec, c = idx % nvec;
      ff2 acc = ZERO;
      for (int k = 0; k < WY_B; ++k) acc = ff_fma(Vs[rr * WY_B + k], Wm[k * nvec + c], acc);
      Zs[rr * nvec + c] = ff_add(Zs[rr * nvec + c], ff_neg(acc));
    }
  }
  __syncthreads();
  for (int idx = tid; idx < nr * nvec; idx += WY_THREADS) {
    const int c = idx / nr, r = idx - c * nr;
    Z[(size_t)c * n + R0 + r] = ff_to_double(Zs[r * nvec + c]);
  }
}

/* evals_desc[i] = w[n-1-i] */
__global__ void k_reverse(const double *w, double *out, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = w[n - 1 - i];
}

/* the pr x pc block grid of k_tridiag_tiled: the largest pr * pc <= G with pr <= pc, both at
 * most TT_MAXG (ties: the smaller pr + pc, so that an index block has fewer parts) */
static void tt_grid(int G, int *pr, int *pc)
{
  int best = 0;
  *pr = *pc = 0;
  for (int r = 1; r * r <= G; ++r) {
    const int c = G / r;
    if (r > TT_MAXG || c > TT_MAXG) continue;
    if (r * c > best || (r * c == best && r + c < *pr + *pc)) {
      best = r * c;
      *pr = r;
      *pc = c;
    }
  }
}

/* the assignment tables of k_tridiag_tiled for every first active tile index J0 (row J0 of
 * rgt [nt][nt] and cgt [nt][nt*TT_UPT]): the active tile rows go to the pr row groups longest
 * first, each to the group with the fewest parts so far (ties: the lower group); then the
 * column units, longest first, each to the column group whose largest block part count grows
 * least (ties: the smaller growth of the sum of squares, then the lower group).  Also the
 * bounds of a block's tile rows, column units and parts over all J0. */
static void tt_tables(int nt, int pr, int pc, std::vector<unsigned char> &rgt,
                      std::vector<unsigned char> &cgt, int *maxr, int *maxc, int *maxi)
{
  const int nu = nt * TT_UPT;
  rgt.assign((size_t)nt * nt, 0);
  cgt.assign((size_t)nt * nu, 0);
  std::vector<int> sum((size_t)pr), L((size_t)pr * pc), suf((size_t)(nt + 1) * pr),
      nrow((size_t)pr), ncol((size_t)pc);
  int mr = 1, mc = 1, mi = 1;
  for (int J0 = 0; J0 < nt; ++J0) {
    unsigned char *rg = &rgt[(size_t)J0 * nt], *cg = &cgt[(size_t)J0 * nu];
    std::fill(sum.begin(), sum.end(), 0);
    for (int I = nt - 1; I >= J0; --I) {
      int best = 0;
      for (int g = 1; g < pr; ++g)
        if (sum[g] < sum[best]) best = g;
      rg[I] = (unsigned char)best;
      sum[best] += TT_UPT * (I - J0 + 1);
    }
    /* suf[J][a]: active tile rows I >= J in row group a (the parts of a unit of tile column J) */
    for (int g = 0; g < pr; ++g) suf[(size_t)nt * pr + g] = 0;
    for (int J = nt - 1; J >= J0; --J) {
      for (int g = 0; g < pr; ++g) suf[(size_t)J * pr + g] = suf[(size_t)(J + 1) * pr + g];
      ++suf[(size_t)J * pr + rg[J]];
    }
    std::fill(L.begin(), L.end(), 0);
    std::fill(ncol.begin(), ncol.end(), 0);
    for (int u = J0 * TT_UPT; u < nu; ++u) {
      const int *v = &suf[(size_t)(u / TT_UPT) * pr];
      int best = 0;
      long long bmax = -1, bsq = 0;
      for (int g = 0; g < pc; ++g) {
        long long mx = 0, sq = 0;
        for (int a = 0; a < pr; ++a) {
          const long long l = L[(size_t)a * pc + g];
          mx = std::max(mx, l + v[a]);
          sq += 2 * l * v[a] + (long long)v[a] * v[a];
        }
        if (bmax < 0 || mx < bmax || (mx == bmax && sq < bsq)) {
          bmax = mx;
          bsq = sq;
          best = g;
        }
      }
      cg[u] = (unsigned char)best;
      ++ncol[best];
      for (int a = 0; a < pr; ++a) L[(size_t)a * pc + best] += v[a];
    }
    std::fill(nrow.begin(), nrow.end(), 0);
    for (int I = J0; I < nt; ++I) ++nrow[rg[I]];
    for (int g = 0; g < pr; ++g) mr = std::max(mr, nrow[g]);
    for (int g = 0; g < pc; ++g) mc = std::max(mc, ncol[g]);
    for (size_t k = 0; k < L.size(); ++k) mi = std::max(mi, L[k]);
  }
  *maxr = mr;
  *maxc = mc;
  *maxi = mi;
}

int gp_eig_tridiag(gp_ctx *ctx, int32_t n, int32_t nvec, double *d_evals_desc, double *d_vecs)
{
  return gp_eig_sym(ctx, ctx->d_xtx, n, nvec, d_evals_desc, d_vecs);
}

/*
 * Eigenpairs of the symmetric n x n device matrix A (overwritten): d_evals_desc [n] all
 * eigenvalues descending, d_vecs [nvec][n] top eigenvectors (descending).  Only this
 * library's kernels run unless the matrix is too large for the cooperative kernels' shared
 * memory (order above 8,533, or a back-transformation slab that does not fit), where cuSOLVER's
 * sytrd / ormtr take over.
 */
int gp_eig_sym(gp_ctx *ctx, double *A_in, int32_t n, int32_t nvec, double *d_evals_desc,
               double *d_vecs)
{
  cusolverDnHandle_t h = ctx->solver;
  int lwork = 0, lwork2 = 0;
  /* GP_EIG_TIMING=1 prints the device time of each stage to stderr */
  const char *tenv = getenv("GP_EIG_TIMING");
  const int timing = tenv && tenv[0] == '1';
  cudaEvent_t ev[7];
  if (timing)
    for (int i = 0; i < 7; ++i) cudaEventCreate(&ev[i]);
#define GP_EIG_MARK(i) \
  if (timing) cudaEventRecord(ev[i], ctx->stream)
  /* scratch: d, e, tau, e2, w, work(sytrd), inverse-iteration work, info */
  int nv = nvec > 0 ? nvec : 1;
  size_t nd = (size_t)n;
  const size_t G = (size_t)ctx->num_sms;
  const size_t nwy = (nd + WY_B - 1) / WY_B;
  /* cuSOLVER workspaces only where its fallbacks can run: the tridiagonalisation above the
   * cooperative kernel's shared memory, or a back-transformation slab that does not fit */
  const size_t rpb0 = (nd + G - 1) / G;
  const size_t q_smem0 = sizeof(double) * (rpb0 * (WY_B + (size_t)nv) + (size_t)WY_B * nv +
                                           WY_B * WY_B + (size_t)WY_B * nv);
  const char *sy_env = getenv("GP_EIG_CUSOLVER_SYTRD"), *or_env = getenv("GP_EIG_CUSOLVER_ORMTR");
  const int may_fallback = n < 2 || 24 * nd > 200 * 1024 || (nvec > 0 && q_smem0 > 200 * 1024) ||
                           (sy_env && sy_env[0] == '1') || (or_env && or_env[0] == '1');
  if (may_fallback) {
    if (cusolverDnDsytrd_bufferSize(h, CUBLAS_FILL_MODE_LOWER, n, A_in, n, NULL, NULL, NULL,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS)
      return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDsytrd_bufferSize failed");
    if (cusolverDnDormtr_bufferSize(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n,
                                    nv, A_in, n, NULL, d_vecs, n, &lwork2) !=
        CUSOLVER_STATUS_SUCCESS)
      return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDormtr_bufferSize failed");
  }
  int lw = lwork > lwork2 ? lwork : lwork2;
  /* partials + sums of k_apply_q, then the blocks' T from k_wy_tmat */
  const size_t qpart_n = (G + 1) * (size_t)WY_B * nv + nwy * WY_B * WY_B;
  size_t bytes = sizeof(double) * (9 * nd + 2 * G + (size_t)lw + 6 * nd * nv + 80 + qpart_n) +
                 sizeof(int) * 64;
  double *base;
  int rc = gp_scratch(ctx, bytes, (void **)&base);
  if (rc) return rc;
  double *d = base, *e = d + nd, *tau = e + nd, *e2 = tau + nd, *w = e2 + nd;
  double *wbuf = w + nd, *ybuf = wbuf + nd, *vbuf = ybuf + 2 * nd, *parts = vbuf + nd;
  unsigned *bar = (unsigned *)(parts + 2 * G);
  double *ws = parts + 2 * G + 16, *iw = ws + lw; /* 16 doubles: barrier words + phase timers */
  int *d_info = (int *)(iw + 6 * nd * nv + 8);
  double *qpart = iw + 6 * nd * nv + 16; /* after d_info's 8 doubles (64 ints) */
  /* the cooperative tridiagonalisation (k_tridiag) unless GP_EIG_CUSOLVER_SYTRD=1, the
   * vectors do not fit shared memory or the device cannot co-schedule one block per SM */
  const char *senv = getenv("GP_EIG_CUSOLVER_SYTRD");
  const size_t tr_smem = 24 * nd;
  int coop = !(senv && senv[0] == '1') && n >= 2 && tr_smem <= 200 * 1024;
  if (coop) {
    int dev_coop = 0, per_sm = 0;
    cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, ctx->device);
    GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_tridiag));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tridiag, TR_THREADS, tr_smem);
    coop = dev_coop && per_sm >= 1;
  }
  /* the lower-triangle tiled variant (k_tridiag_tiled) where its shared memory fits, unless
   * GP_TRIDIAG_TILED=0; the whole-matrix k_tridiag otherwise */
  const char *tt_env = getenv("GP_TRIDIAG_TILED");
  const int nt = (n + TT - 1) / TT;
  int tt_pr = 0, tt_pc = 0, tt_maxr = 0, tt_maxc = 0, tt_maxi = 0;
  size_t tt_smem = 0;
  /* the tiled steps run while the trailing order exceeds tt_switch (GP_TRIDIAG_SWITCH), where
   * the whole-column steps, with more rows per block than tile rows, take over */
  const char *sw_env = getenv("GP_TRIDIAG_SWITCH");
  const int tt_switch = sw_env && sw_env[0] ? atoi(sw_env) : 2500;
  const int tt_cs = n - 1 - std::max(1, tt_switch); /* first whole-column step */
  int tiled = !(senv && senv[0] == '1') && !(tt_env && tt_env[0] == '0') && tt_cs >= 1 &&
              tr_smem <= 200 * 1024;
  if (tiled) {
    tt_grid((int)G, &tt_pr, &tt_pc);
    tiled = tt_pr >= 1 && tt_pc >= 1;
  }
  int tt_R = 0;
  if (tiled && !(ctx->d_tt && ctx->tt_n == n && ctx->tt_G == (int)G)) {
    /* the assignment tables, once per order and grid */
    std::vector<unsigned char> rgt, cgt;
    tt_tables(nt, tt_pr, tt_pc, rgt, cgt, &ctx->tt_maxr, &ctx->tt_maxc, &ctx->tt_maxi);
    ctx->tt_n = 0;
    int rc3 = gp_realloc(ctx, (void **)&ctx->d_tt, rgt.size() + cgt.size());
    if (rc3) return rc3;
    GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_tt, rgt.data(), rgt.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
    GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_tt + rgt.size(), cgt.data(), cgt.size(),
                           cudaMemcpyHostToDevice, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->tt_n = n;
    ctx->tt_G = (int)G;
  }
  if (tiled) {
    tt_maxr = ctx->tt_maxr;
    tt_maxc = ctx->tt_maxc;
    tt_maxi = ctx->tt_maxi;
    /* parts per round: all of a block's parts in one round where shared memory allows
     * (GP_TT_ROUND caps it, to run the several-round path at smaller orders) */
    tt_R = std::min(128, (tt_maxi + TR_WARPS - 1) / TR_WARPS * TR_WARPS);
    const char *r_env = getenv("GP_TT_ROUND");
    if (r_env && atoi(r_env) >= TR_WARPS)
      tt_R = std::min(tt_R, atoi(r_env) / TR_WARPS * TR_WARPS);
    while (tt_R > TR_WARPS && tt_smem_bytes(nt, tt_R, tt_maxr, tt_maxc, tt_maxi) > 220 * 1024)
      tt_R -= TR_WARPS;
    tt_smem = tt_smem_bytes(nt, tt_R, tt_maxr, tt_maxc, tt_maxi);
    tiled = tt_maxr <= 512 && tt_maxc <= 512 && tt_smem <= 220 * 1024;
  }
  if (tiled) {
    int dev_coop = 0, per_sm = 0;
    cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, ctx->device);
    tiled = dev_coop && gp_allow_smem(ctx, (const void *)k_tridiag_tiled) == cudaSuccess;
    if (tiled) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tridiag_tiled, TR_THREADS,
                                                    tt_smem);
      tiled = per_sm >= 1;
    }
    (void)cudaGetLastError();
  }
  if (tiled) coop = 1;
  if (!coop && !may_fallback)
    return gp_fail(ctx, GP_ERR_CUDA, "eigensolve: the cooperative tridiagonalisation cannot run");
  GP_EIG_MARK(0);
  int info = 0;
  if (tiled) {
    const int64_t ntiles = (int64_t)nt * (nt + 1) / 2;
    const size_t tile_d = (size_t)ntiles * TT * TT;
    const size_t part_d = (size_t)(tt_pr + tt_pc) * nt * TT; /* prow + pcol */
    const size_t tri_bytes = sizeof(double) * (tile_d + part_d + 2 * (size_t)nt) +
                             sizeof(unsigned) * (size_t)nt;
    int rc2 = gp_realloc(ctx, (void **)&ctx->d_tri, tri_bytes);
    if (rc2) return rc2;
    double *Tm = ctx->d_tri, *prow = Tm + tile_d, *pcol = prow + (size_t)nt * tt_pc * TT;
    double *dotp = pcol + (size_t)nt * tt_pr * TT;
    unsigned *kcnt = (unsigned *)(dotp + 2 * (size_t)nt);
    int *d_err = ctx->d_err;
    GP_CUDA(ctx, cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
    GP_CUDA(ctx, cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), ctx->stream));
    GP_CUDA(ctx, cudaMemsetAsync(kcnt, 0, sizeof(unsigned) * (size_t)nt, ctx->stream));
    {
      int blocks = (int)std::min<int64_t>(ntiles, (int64_t)ctx->num_sms * 8);
      k_tri_to_tiles<<<blocks, 256, 0, ctx->stream>>>(A_in, n, nt, Tm);
      GP_LAUNCH_CHECK(ctx, "k_tri_to_tiles");
    }
    unsigned long long *phase = NULL;
    if (timing) {
      phase = (unsigned long long *)(bar + 8);
      GP_CUDA(ctx, cudaMemsetAsync(phase, 0, 5 * sizeof(unsigned long long), ctx->stream));
    }
    double *A = A_in, *pd2 = parts;
    int nn = n, nt_ = nt, cs = tt_cs;
    const unsigned char *rgt = ctx->d_tt, *cgt = ctx->d_tt + (size_t)nt * nt;
    void *args[] = {&A,    &Tm,   &nn,   &nt_,  &tt_pr, &tt_pc, &tt_maxr, &tt_maxc,
                    &tt_maxi, &tt_R, &cs, &rgt, &cgt,  &d,     &e,       &tau,
                    &vbuf, &wbuf, &ybuf, &prow, &pcol, &dotp,  &kcnt,    &pd2,
                    &bar,  &d_err, &phase};
    GP_CUDA(ctx, cudaEventRecord(ctx->ev_tr0, ctx->stream));
    GP_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)k_tridiag_tiled, dim3((unsigned)G),
                                             dim3(TR_THREADS), args, tt_smem, ctx->stream));
    GP_CUDA(ctx, cudaEventRecord(ctx->ev_tr1, ctx->stream));
    ctx->launches++;
    int herr = 0;
    GP_CUDA(ctx, gp_memcpy(ctx, &herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (herr == TR_ERR_LISTS)
      return gp_fail(ctx, GP_ERR_CUDA, "tiled tridiagonalisation: a block's tile lists overflowed");
    if (herr == TR_ERR_WAIT)
      return gp_fail(ctx, GP_ERR_TIMEOUT, "tiled tridiagonalisation: an index block's parts "
                                          "did not arrive in time");
    if (herr) return gp_fail(ctx, GP_ERR_TIMEOUT, "tridiagonalisation grid barrier timed out");
    float tms = 0.f;
    GP_CUDA(ctx, cudaEventElapsedTime(&tms, ctx->ev_tr0, ctx->ev_tr1));
    if (A_in == ctx->d_xtx) {
      ctx->tridiag_ms = tms;
      ctx->tridiag_n = n;
    }
    if (timing) {
      unsigned long long hp[5];
      cudaMemcpy(hp, phase, sizeof hp, cudaMemcpyDeviceToHost);
      fprintf(stderr,
              "k_tridiag_tiled n=%d grid %dx%d, whole columns from step %d (block 0): A %.1f ms, "
              "B %.1f (first 30%% of steps %.1f), barrier %.1f\n",
              n, tt_pr, tt_pc, tt_cs, hp[0] * 1e-6, (hp[1] + hp[2]) * 1e-6, hp[2] * 1e-6,
              hp[4] * 1e-6);
    }
  } else if (coop) {
    int *d_err = ctx->d_err;
    GP_CUDA(ctx, cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
    GP_CUDA(ctx, cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), ctx->stream));
    double *A = A_in, *pd2 = parts;
    int nn = n;
    {
      int64_t tot = (int64_t)n * n;
      int blocks = (int)((tot + 255) / 256);
      if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
      k_tri_to_ff<<<blocks, 256, 0, ctx->stream>>>(A, n);
      GP_LAUNCH_CHECK(ctx, "k_tri_to_ff");
    }
    unsigned long long *phase = NULL;
    if (timing) {
      phase = (unsigned long long *)(bar + 8);
      GP_CUDA(ctx, cudaMemsetAsync(phase, 0, 5 * sizeof(unsigned long long), ctx->stream));
    }
    void *args[] = {&A, &nn, &d, &e, &tau, &vbuf, &wbuf, &ybuf, &pd2, &bar, &d_err, &phase};
    GP_CUDA(ctx, cudaEventRecord(ctx->ev_tr0, ctx->stream));
    GP_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)k_tridiag, dim3((unsigned)G),
                                             dim3(TR_THREADS), args, tr_smem, ctx->stream));
    GP_CUDA(ctx, cudaEventRecord(ctx->ev_tr1, ctx->stream));
    ctx->launches++;
    int herr = 0;
    GP_CUDA(ctx, gp_memcpy(ctx, &herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (herr) return gp_fail(ctx, GP_ERR_TIMEOUT, "tridiagonalisation grid barrier timed out");
    float tms = 0.f;
    GP_CUDA(ctx, cudaEventElapsedTime(&tms, ctx->ev_tr0, ctx->ev_tr1));
    if (A_in == ctx->d_xtx) { /* the Gram's eigensolve: its time is reported */
      ctx->tridiag_ms = tms;
      ctx->tridiag_n = n;
    }
    if (timing) {
      unsigned long long hp[5];
      cudaMemcpy(hp, phase, sizeof hp, cudaMemcpyDeviceToHost);
      fprintf(stderr,
              "k_tridiag n=%d (block 0): A %.1f ms, B %.1f (first 30%% of steps %.1f), "
              "barrier %.1f\n",
              n, hp[0] * 1e-6, (hp[1] + hp[2]) * 1e-6, hp[2] * 1e-6, hp[4] * 1e-6);
    }
  } else {
    ctx->tridiag_ms = 0.0;
    ctx->tridiag_n = n;
    if (cusolverDnDsytrd(h, CUBLAS_FILL_MODE_LOWER, n, A_in, n, d, e, tau, ws, lw,
                         d_info) != CUSOLVER_STATUS_SUCCESS)
      return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDsytrd failed to launch");
    GP_CUDA(ctx, gp_memcpy(ctx, &info, d_info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  }
  GP_EIG_MARK(1);
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
    /* GP_EIG_NO_FF=1 selects the path without the float-float phase (as for N > 6,400) */
    const char *ffenv = getenv("GP_EIG_NO_FF");
    size_t smem = (size_t)32 * (size_t)n;
    int use_smem = 2;
    if (smem > 200 * 1024 || (ffenv && ffenv[0] == '1')) {
      smem = (size_t)24 * (size_t)n;
      use_smem = smem <= 200 * 1024 ? 1 : 0;
    }
    const int warps = ctx->num_sms * 4;
    int epw = (n + warps - 1) / warps;
    if (epw > 32) epw = 32;
    const int P = 32 / epw;
    const int nwarps = (n + epw - 1) / epw;
    const int blocks = (nwarps + 3) / 4;
    /* FP64 brackets end at 1e-13 ||T||: the counts' own backward error is ~6e-14 ||T|| */
    const double tol = 1e-13 * tnorm;
    if (use_smem)
      GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_multisect));
    k_multisect<<<blocks, 128, use_smem ? smem : 0, ctx->stream>>>(d, e2, n, gl, gu, tnorm, pivmin,
                                                                   tol, use_smem, epw, P, w);
    GP_LAUNCH_CHECK(ctx, "k_multisect");
  }
  k_reverse<<<(n + 255) / 256, 256, 0, ctx->stream>>>(w, d_evals_desc, n);
  GP_LAUNCH_CHECK(ctx, "k_reverse");
  GP_EIG_MARK(3);
  if (nvec > 0) {
    /* factors, iterate and byte pivots: 41 n bytes */
    const size_t ii_smem = (size_t)n * (5 * sizeof(double) + 1) + 16;
    int smem_optin = 0;
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    /* GP_EIG_II_GLOBAL=1 selects the global-memory path (as for N > 5,600) */
    const char *iienv = getenv("GP_EIG_II_GLOBAL");
    const int ii_in_smem = ii_smem + 2048 <= (size_t)smem_optin && !(iienv && iienv[0] == '1');
    if (ii_in_smem)
      GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_inverse_iteration));
    k_inverse_iteration<<<nvec, 256, ii_in_smem ? ii_smem : 0, ctx->stream>>>(
        d, e, n, w, nvec, tnorm, d_vecs, iw, ii_in_smem);
    GP_LAUNCH_CHECK(ctx, "k_inverse_iteration");
    GP_EIG_MARK(5);
    k_mgs<<<1, 1024, 0, ctx->stream>>>(d_vecs, n, nvec);
    GP_LAUNCH_CHECK(ctx, "k_mgs");
    GP_EIG_MARK(6);
    /* Z := Q Z: the cooperative WY kernel when its row slab fits shared memory, else
     * cusolverDnDormtr (GP_EIG_CUSOLVER_ORMTR=1 forces the latter) */
    const char *oenv = getenv("GP_EIG_CUSOLVER_ORMTR");
    const int Gq = ctx->num_sms;
    const size_t rpb = ((size_t)n + Gq - 1) / Gq;
    const size_t nent = (size_t)WY_B * nvec;
    const size_t q_smem = sizeof(double) * (rpb * (WY_B + nvec) + nent + WY_B * WY_B + (size_t)WY_B * nvec);
    int qcoop = !(oenv && oenv[0] == '1') && n >= 2 && q_smem <= 200 * 1024 &&
                qpart != NULL;
    if (qcoop) {
      int dev_coop = 0, per_sm = 0;
      cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, ctx->device);
      GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_apply_q));
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_q, WY_THREADS, q_smem);
      qcoop = dev_coop && per_sm >= 1;
    }
    if (!qcoop && !may_fallback)
      return gp_fail(ctx, GP_ERR_CUDA, "eigensolve: the cooperative back-transformation cannot run");
    if (qcoop) {
      unsigned *qbar = bar + 4;
      int *d_err = ctx->d_err;
      GP_CUDA(ctx, cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
      GP_CUDA(ctx, cudaMemsetAsync(qbar, 0, sizeof(unsigned), ctx->stream));
      const double *Aq = A_in;
      double *Sq = qpart + (size_t)Gq * nent;
      double *Tg = qpart + (size_t)(Gq + 1) * nent;
      const int nwyb = (n - 1 + WY_B - 1) / WY_B;
      k_wy_tmat<<<nwyb, WT_THREADS, 0, ctx->stream>>>(Aq, n, tau, Tg);
      GP_LAUNCH_CHECK(ctx, "k_wy_tmat");
      const double *Tgc = Tg;
      int nn = n, nv2 = nvec;
      void *qargs[] = {(void *)&Aq, &nn, (void *)&Tgc, &d_vecs, &nv2, &qpart, &Sq, &qbar, &d_err};
      GP_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)k_apply_q, dim3((unsigned)Gq),
                                               dim3(WY_THREADS), qargs, q_smem, ctx->stream));
      ctx->launches++;
      int herr = 0;
      GP_CUDA(ctx, gp_memcpy(ctx, &herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (herr) return gp_fail(ctx, GP_ERR_TIMEOUT, "back-transformation grid barrier timed out");
    } else {
      if (cusolverDnDormtr(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, nvec,
                           A_in, n, tau, d_vecs, n, ws, lw, d_info) != CUSOLVER_STATUS_SUCCESS)
        return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDormtr failed to launch");
      GP_CUDA(ctx, gp_memcpy(ctx, &info, d_info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (info != 0) return gp_fail(ctx, GP_ERR_SOLVER, "ormtr info = %d", info);
    }
  }
  if (timing) {
    GP_EIG_MARK(4);
    cudaEventSynchronize(ev[4]);
    float t01 = 0, t23 = 0, t34 = 0, t35 = 0, t56 = 0;
    cudaEventElapsedTime(&t01, ev[0], ev[1]);
    cudaEventElapsedTime(&t23, ev[2], ev[3]);
    cudaEventElapsedTime(&t34, ev[3], ev[4]);
    if (nvec > 0) {
      cudaEventElapsedTime(&t35, ev[3], ev[5]);
      cudaEventElapsedTime(&t56, ev[5], ev[6]);
    }
    fprintf(stderr, "eig n=%d: tridiagonal %.1f ms, eigenvalues %.1f ms, vectors %.1f ms "
            "(inverse iteration %.1f, mgs %.1f)\n", n, t01, t23, t34, t35, t56);
    for (int i = 0; i < 7; ++i) cudaEventDestroy(ev[i]);
  }
  return GP_OK;
}
