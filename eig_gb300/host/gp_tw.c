/*
 * Tracy-Widom statistics of smartpca's log (src/eigensrc/smartpca.c:1312-1367) and the
 * mpstats line before them (mpestimate, smartpca.c:4532-4560), restated on the host.
 *
 * For eigenvalue i of the m positive ones, dotwcalc (src/nicksrc/statsubs.c:1680-1725) scales
 * lambda[i..m-1] to mean 1, takes the effective number of markers n' = m(m+2) / (sum l^2 - m)
 * (Patterson, Price & Reich 2006, appendix), normalises the top value with Johnstone's (2001)
 * centring and scaling (twnorm, statsubs.c:1658-1677) and reports the right tail of the
 * Tracy-Widom distribution TW1 there.  The reference reads that tail from a compiled-in table
 * of TW1 on x = -8.0, -7.9, ..., 8.0 (tail and density) and interpolates it with a cubic
 * Hermite polynomial (gettw / cinterp, statsubs.c:1811-1905); below the table the tail is 1,
 * and at or above its last point it returns the Margetis-Edelman asymptotic DENSITY in place
 * of the tail (the two outputs of twdensx / twtailx are swapped there), which is kept.
 *
 * The table is not copied: this file computes TW1 itself on the same grid, from the Fredholm
 * determinant F1(s) = det(I - K_s) on L2(0, inf) with K_s(x, y) = Ai(x + y + s)
 * (Ferrari & Spohn 2005), discretised by Gauss-Legendre quadrature as in Bornemann,
 * "On the numerical evaluation of Fredholm determinants", Math. Comp. 79 (2010) 871-915.
 * The density follows from Jacobi's formula, d/ds log det(I - K) = -tr((I - K)^-1 dK/ds) with
 * dK/ds(x, y) = Ai'(x + y + s).  Where K is small (s >= 3) log det(I - K) is summed as
 * -sum_n tr(K^n)/n, so that a small tail keeps its relative accuracy; elsewhere an LU
 * factorisation with partial pivoting gives the determinant and the solve.
 *
 * Ai and Ai' are the Maclaurin series for -7 <= x <= 5 and the classical asymptotic
 * expansions outside (Abramowitz & Stegun 10.4.58-10.4.63: the exponentially decaying one for
 * x > 5, the oscillatory one for x < -7, coefficients u_k = (6k-5)(6k-3)(6k-1) u_{k-1} /
 * ((2k-1) 216 k), v_k = -(6k+1)/(6k-1) u_k), each summed to below 1e-17 or to its smallest
 * term.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gpupca_run.h"

#define TW_GRID_N 161
#define TW_GRID_X0 (-8.0)
#define TW_GRID_DX 0.1
#define TW_QUAD 64
#define TW_SERIES_S 3.0 /* log det by its trace series from here on (K small) */

/* Ai(x) and Ai'(x) */
static void airy(double x, double *ai, double *aip)
{
  const double c1 = 0.355028053887817239260; /* Ai(0) = 1 / (3^(2/3) Gamma(2/3)) */
  const double c2 = 0.258819403792806798405; /* -Ai'(0) = 1 / (3^(1/3) Gamma(1/3)) */
  const double sqpi = 1.772453850905516027298;
  if (x >= -7.0 && x <= 5.0) {
    /* f = sum a_k x^3k, g = sum b_k x^(3k+1), a_k = a_(k-1) / (3k (3k-1)),
     * b_k = b_(k-1) / (3k (3k+1)); Ai = c1 f - c2 g */
    const double x3 = x * x * x;
    double a = 1.0, b = x, f = 1.0, g = x, fp = 0.0, gp = 1.0;
    for (int k = 1; k < 200; ++k) {
      a *= x3 / ((3.0 * k) * (3.0 * k - 1.0));
      b *= x3 / ((3.0 * k) * (3.0 * k + 1.0));
      f += a;
      g += b;
      /* derivatives: d/dx a_k x^3k = 3k a_k x^(3k-1); d/dx b_k x^(3k+1) = (3k+1) b_k x^3k */
      fp += (x != 0.0) ? 3.0 * k * a / x : 0.0;
      gp += (x != 0.0) ? (3.0 * k + 1.0) * b / x : 0.0;
      if (fabs(a) + fabs(b) < 1e-18 * (fabs(f) + fabs(g)) && k > 2) break;
    }
    *ai = c1 * f - c2 * g;
    *aip = c1 * fp - c2 * gp;
    return;
  }
  if (x > 5.0) {
    const double z = sqrt(x), zeta = 2.0 / 3.0 * x * z, e = exp(-zeta);
    double u = 1.0, v = 1.0, su = 1.0, sv = 1.0, t = 1.0, last = 1.0;
    for (int k = 1; k < 60; ++k) {
      u *= (6.0 * k - 5.0) * (6.0 * k - 3.0) * (6.0 * k - 1.0) / ((2.0 * k - 1.0) * 216.0 * k);
      v = -(6.0 * k + 1.0) / (6.0 * k - 1.0) * u;
      t /= -zeta;
      const double tu = u * t;
      if (fabs(tu) > last) break; /* past the smallest term */
      last = fabs(tu);
      su += tu;
      sv += v * t;
      if (last < 1e-18) break;
    }
    const double q = sqrt(sqrt(x));
    *ai = e / (2.0 * sqpi * q) * su;
    *aip = -q * e / (2.0 * sqpi) * sv;
    return;
  }
  /* x < -7: Ai(-z) = pi^-1/2 z^-1/4 [sin(zeta + pi/4) P - cos(zeta + pi/4) Q],
   * Ai'(-z) = -pi^-1/2 z^1/4 [cos(zeta + pi/4) R + sin(zeta + pi/4) S] */
  {
    const double zz = -x, z = sqrt(zz), zeta = 2.0 / 3.0 * zz * z;
    double P = 1.0, Q = 0.0, R = 1.0, S = 0.0, u = 1.0, v = 1.0, t = 1.0, last = 1.0;
    for (int k = 1; k < 60; ++k) {
      u *= (6.0 * k - 5.0) * (6.0 * k - 3.0) * (6.0 * k - 1.0) / ((2.0 * k - 1.0) * 216.0 * k);
      v = -(6.0 * k + 1.0) / (6.0 * k - 1.0) * u;
      t /= zeta;
      const double tu = u * t;
      if (fabs(tu) > last) break;
      last = fabs(tu);
      /* k even: P, R get (-1)^(k/2) terms; k odd: Q, S get (-1)^((k-1)/2) terms */
      const double sg = ((k / 2) % 2 == 0) ? 1.0 : -1.0;
      if (k % 2 == 0) {
        P += sg * tu;
        R += sg * v * t;
      } else {
        Q += sg * tu;
        S += sg * v * t;
      }
      if (last < 1e-18) break;
    }
    const double ph = zeta + 0.25 * M_PI, sn = sin(ph), cs = cos(ph);
    const double q = sqrt(z);
    *ai = (sn * P - cs * Q) / (sqpi * q);
    *aip = -q * (cs * R + sn * S) / sqpi;
  }
}

/* Gauss-Legendre nodes and weights on [0, L] (Newton on the Legendre recurrence) */
static void gauss_legendre(int m, double L, double *x, double *w)
{
  for (int i = 0; i < (m + 1) / 2; ++i) {
    double z = cos(M_PI * (i + 0.75) / (m + 0.5)), pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= m; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = m * (z * p1 - p2) / (z * z - 1.0);
      const double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    const double wi = 2.0 / ((1.0 - z * z) * pp * pp);
    x[i] = 0.5 * L * (1.0 - z);
    x[m - 1 - i] = 0.5 * L * (1.0 + z);
    w[i] = w[m - 1 - i] = 0.5 * L * wi;
  }
}

/* F1(s) = det(I - K_s), its right tail 1 - F1 and density F1'(s) */
static void tw1(double s, double *tail, double *dens)
{
  const int m = TW_QUAD;
  double x[TW_QUAD], w[TW_QUAD], sw[TW_QUAD];
  const double L = s < 16.0 ? 16.0 - s : 4.0;
  gauss_legendre(m, L, x, w);
  for (int i = 0; i < m; ++i) sw[i] = sqrt(w[i]);
  double *K = (double *)malloc(sizeof(double) * m * m * 4);
  double *Kp = K + m * m, *T1 = Kp + m * m, *T2 = T1 + m * m;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      double a, ap;
      airy(x[i] + x[j] + s, &a, &ap);
      K[i * m + j] = sw[i] * a * sw[j];
      Kp[i * m + j] = sw[i] * ap * sw[j];
    }
  double logdet = 0.0, dlog = 0.0; /* log det(I - K), d/ds of it */
  if (s >= TW_SERIES_S) {
    /* -sum tr(K^n)/n and -sum tr(K^(n-1) K'): T1 = K^(n-1), T2 = K^(n-1) K' */
    for (int i = 0; i < m * m; ++i) T1[i] = 0.0;
    for (int i = 0; i < m; ++i) T1[i * m + i] = 1.0;
    for (int n = 1; n < 400; ++n) {
      double trk = 0.0, trd = 0.0;
      for (int i = 0; i < m; ++i)
        for (int k = 0; k < m; ++k) {
          trk += T1[i * m + k] * K[k * m + i];
          trd += T1[i * m + k] * Kp[k * m + i];
        }
      logdet -= trk / n;
      dlog -= trd;
      if (fabs(trk) / n < 1e-19 * (fabs(logdet) + 1e-300) && fabs(trd) < 1e-19 * fabs(dlog)) break;
      for (int i = 0; i < m; ++i) /* T1 <- T1 K */
        for (int j = 0; j < m; ++j) {
          double acc = 0.0;
          for (int k = 0; k < m; ++k) acc += T1[i * m + k] * K[k * m + j];
          T2[i * m + j] = acc;
        }
      memcpy(T1, T2, sizeof(double) * m * m);
    }
  } else {
    /* LU with partial pivoting of A = I - K, then tr(A^-1 K') from the solves */
    double *A = T1;
    int piv[TW_QUAD];
    for (int i = 0; i < m * m; ++i) A[i] = -K[i];
    for (int i = 0; i < m; ++i) A[i * m + i] += 1.0;
    for (int c = 0; c < m; ++c) {
      int p = c;
      for (int r = c + 1; r < m; ++r)
        if (fabs(A[r * m + c]) > fabs(A[p * m + c])) p = r;
      piv[c] = p;
      if (p != c)
        for (int j = 0; j < m; ++j) {
          const double t = A[c * m + j];
          A[c * m + j] = A[p * m + j];
          A[p * m + j] = t;
        }
      logdet += log(fabs(A[c * m + c]));
      for (int r = c + 1; r < m; ++r) {
        const double l = A[r * m + c] / A[c * m + c];
        A[r * m + c] = l;
        for (int j = c + 1; j < m; ++j) A[r * m + j] -= l * A[c * m + j];
      }
    }
    /* column j of A^-1 K': P A = L U with the row interchanges applied to whole rows, so the
     * right-hand side takes all of them in order before the forward substitution */
    double col[TW_QUAD];
    for (int j = 0; j < m; ++j) {
      for (int i = 0; i < m; ++i) col[i] = Kp[i * m + j];
      for (int c = 0; c < m; ++c) {
        const int p = piv[c];
        if (p != c) {
          const double t = col[c];
          col[c] = col[p];
          col[p] = t;
        }
      }
      for (int c = 0; c < m; ++c)
        for (int r = c + 1; r < m; ++r) col[r] -= A[r * m + c] * col[c];
      for (int c = m - 1; c >= 0; --c) {
        double acc = col[c];
        for (int k = c + 1; k < m; ++k) acc -= A[c * m + k] * col[k];
        col[c] = acc / A[c * m + c];
      }
      dlog -= col[j];
    }
  }
  free(K);
  const double F = exp(logdet);
  *tail = -expm1(logdet);
  *dens = F * dlog; /* F1' = F1 d/ds log F1 */
}

static double tw_x[TW_GRID_N], tw_tail_tab[TW_GRID_N], tw_dens_tab[TW_GRID_N];
static pthread_once_t tw_once = PTHREAD_ONCE_INIT;

static void tw_build(void)
{
  for (int k = 0; k < TW_GRID_N; ++k) {
    tw_x[k] = TW_GRID_X0 + TW_GRID_DX * k;
    tw_x[k] = round(tw_x[k] * 10.0) / 10.0;
    tw1(tw_x[k], &tw_tail_tab[k], &tw_dens_tab[k]);
  }
}

/* the table, built once per process (callers on several threads wait for the first) */
static void tw_table(void) { pthread_once(&tw_once, tw_build); }

/* the reference's bisection for the first table entry above val (statsubs.c:1745-1764) */
static int first_above(const double *tab, int lo, int hi, double val)
{
  if (val >= tab[hi]) return hi + 1;
  if (val < tab[lo]) return lo;
  const int k = (lo + hi) / 2;
  if (val <= tab[k]) return first_above(tab, lo + 1, k, val);
  return first_above(tab, k, hi - 1, val);
}

double gp_tw_tail(double x)
{
  tw_table();
  const int n = TW_GRID_N;
  const int k = first_above(tw_x, 0, n - 1, x);
  if (k <= 0) return 1.0;
  if (k >= n) {
    /* the Margetis-Edelman density, as the reference's table lookup returns past its end */
    if (x <= 0.0) return 0.0;
    return exp(-0.25 * log(x) - 2.0 * pow(x, 1.5) / 3.0 - log(4.0 * sqrt(M_PI)));
  }
  /* cubic Hermite interpolation of the tail (derivative minus the density) */
  const double x0 = tw_x[k - 1], x1 = tw_x[k], inc = x1 - x0, y = (x - x0) / inc;
  const double a0 = tw_tail_tab[k - 1], a1 = -tw_dens_tab[k - 1] * inc;
  const double cc0 = tw_tail_tab[k] - (a0 + a1), cc1 = -tw_dens_tab[k] * inc - a1;
  const double a2 = 3 * cc0 - cc1, a3 = cc1 - 2 * cc0;
  return ((a3 * y + a2) * y + a1) * y + a0;
}

/* Johnstone's normalisation of the top eigenvalue (symmetric in p and n - 1) */
static double tw_norm(double lam, double p, double n)
{
  if (n < 0.0 || p < 0.0) return -10.0;
  if (n < p) return tw_norm(lam, n, p);
  const double y1 = sqrt(n - 1.0) + sqrt(p), mu = y1 * y1;
  const double y2 = 1.0 / sqrt(n - 1.0) + 1.0 / sqrt(p);
  const double phi = y1 * pow(y2, 1.0 / 3.0);
  return (lam - mu) / phi;
}

int gp_twstats(const double *lambda, int32_t m, int32_t nrows, double znval,
               int32_t nostatslim, double *twstat, double *pvalue, double *effn)
{
  if (!lambda || m < 0 || !twstat || !pvalue || !effn) return GP_ERR_ARG;
  const double ynrows = (double)nrows;
  for (int32_t i = 0; i < m; ++i) {
    const double *lam = lambda + i;
    const int32_t len = m - i;
    double zn = znval;
    if (zn > 0.0) zn = zn > ynrows ? zn : ynrows;
    twstat[i] = pvalue[i] = effn[i] = -1.0;
    if (len < nostatslim) continue;
    double lsum = 0.0;
    for (int32_t k = 0; k < len; ++k) lsum += lam[k];
    if (lsum <= 0.0) continue;
    const double y = (double)len / lsum;
    if (zn > 0.0) {
      twstat[i] = tw_norm(lam[0] * y * zn, (double)len, zn);
      effn[i] = zn;
    } else {
      double s2 = 0.0;
      for (int32_t k = 0; k < len; ++k) {
        const double e = lam[k] * y;
        s2 += e * e;
      }
      const double z = (double)len * (double)(len + 2) / (s2 - (double)len);
      twstat[i] = tw_norm(lam[0] * y * z, (double)len, z);
      effn[i] = z;
    }
    pvalue[i] = gp_tw_tail(twstat[i]);
  }
  return GP_OK;
}

/* the reference's quartile: linear interpolation of the sorted values at index q (n - 1)
 * (quartile / qinterp, statsubs.c:2998-3090) */
static int cmp_double(const void *a, const void *b)
{
  const double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

static double quartile(const double *sorted, int n, double q)
{
  if (n == 1) return sorted[0];
  /* sentinel-extended index axis -1e20, 0, 1, ..., n-1, n-1+1e20 and the sorted values */
  double *xa = (double *)malloc(sizeof(double) * (size_t)(n + 2));
  xa[0] = 0.0 - 1.0e20;
  for (int k = 0; k < n; ++k) xa[k + 1] = (double)k;
  xa[n + 1] = (double)(n - 1) + 1.0e20;
  const double val = q * (double)(n - 1);
  const int x = first_above(xa, 0, n + 1, val);
  double ans;
  if (x <= 1) {
    ans = sorted[0];
  } else if (x == n + 1) {
    ans = sorted[n - 1];
  } else {
    double y1 = xa[x] - val, y2 = val - xa[x - 1];
    const double yy = y1 + y2;
    y1 /= yy;
    y2 /= yy;
    const double b0 = sorted[x - 2], b1 = (x - 1 < n) ? sorted[x - 1] : sorted[n - 1];
    ans = y1 * b0 + y2 * b1;
  }
  free(xa);
  return ans;
}

int gp_mpstats(const double *lambda, int32_t m, double *out4)
{
  if (!lambda || !out4) return GP_ERR_ARG;
  if (m < 10) return 1;
  double *s = (double *)malloc(sizeof(double) * (size_t)m);
  if (!s) return GP_ERR_NOMEM;
  memcpy(s, lambda, sizeof(double) * (size_t)m);
  qsort(s, (size_t)m, sizeof(double), cmp_double);
  out4[0] = quartile(s, m, 0.25);
  out4[1] = quartile(s, m, 0.50);
  out4[2] = quartile(s, m, 0.75);
  out4[3] = (out4[2] - out4[0]) / out4[1];
  free(s);
  return GP_OK;
}
