/*
 * Tail probabilities of smartpca's ANOVA tail (dottest / publishit / popdifference,
 * src/eigensrc/smartpca.c:2316-2572 and :1977-1993), written from the mathematics:
 *
 *   F upper tail      Q(F | d1, d2) = I_x(d2/2, d1/2), x = d2 / (d2 + d1 F)
 *   chi-square tail   Q(z | d) = Q(d/2, z/2) (regularised upper incomplete gamma);
 *                     d = 1: erfc(sqrt(z/2)); d = 2: exp(-z/2)
 *
 * with the regularised incomplete beta and gamma functions evaluated by the modified Lentz
 * continued fractions (and the power series of P(a, x) below x = a + 1), as published in
 * Press, Teukolsky, Vetterling & Flannery, Numerical Recipes, 2nd ed., sections 6.2 and 6.4.
 */
#include "gp_stats.h"

#include <float.h>
#include <math.h>

#define CF_EPS 1.0e-16
#define CF_TINY 1.0e-300
#define CF_MAXIT 10000

/* continued fraction of I_x(a, b) (the even and odd steps d_2m, d_2m+1) */
static double beta_cf(double a, double b, double x)
{
  double c = 1.0, d = 1.0 - (a + b) * x / (a + 1.0);
  if (fabs(d) < CF_TINY) d = CF_TINY;
  d = 1.0 / d;
  double h = d;
  for (int m = 1; m <= CF_MAXIT; ++m) {
    const double m2 = 2.0 * m;
    double aa = m * (b - m) * x / ((a + m2 - 1.0) * (a + m2));
    d = 1.0 + aa * d;
    if (fabs(d) < CF_TINY) d = CF_TINY;
    c = 1.0 + aa / c;
    if (fabs(c) < CF_TINY) c = CF_TINY;
    d = 1.0 / d;
    h *= d * c;
    aa = -(a + m) * (a + b + m) * x / ((a + m2) * (a + m2 + 1.0));
    d = 1.0 + aa * d;
    if (fabs(d) < CF_TINY) d = CF_TINY;
    c = 1.0 + aa / c;
    if (fabs(c) < CF_TINY) c = CF_TINY;
    d = 1.0 / d;
    const double del = d * c;
    h *= del;
    if (fabs(del - 1.0) < CF_EPS) break;
  }
  return h;
}

double gp_betai(double a, double b, double x)
{
  if (x <= 0.0) return 0.0;
  if (x >= 1.0) return 1.0;
  const double lbt = lgamma(a + b) - lgamma(a) - lgamma(b) + a * log(x) + b * log1p(-x);
  if (x < (a + 1.0) / (a + b + 2.0)) return exp(lbt) * beta_cf(a, b, x) / a;
  return 1.0 - exp(lbt) * beta_cf(b, a, 1.0 - x) / b;
}

double gp_gammq(double a, double x)
{
  if (x <= 0.0) return 1.0;
  const double lpre = a * log(x) - x - lgamma(a);
  if (x < a + 1.0) {
    /* P(a, x) = e^-x x^a / Gamma(a+1) * sum x^n / ((a+1)...(a+n)) */
    double ap = a, del = 1.0 / a, sum = del;
    for (int n = 0; n < CF_MAXIT; ++n) {
      ap += 1.0;
      del *= x / ap;
      sum += del;
      if (fabs(del) < fabs(sum) * CF_EPS) break;
    }
    return 1.0 - sum * exp(lpre);
  }
  /* Q(a, x) = e^-x x^a / Gamma(a) * 1 / (x + 1 - a - 1 (1 - a) / (x + 3 - a - ...)) */
  double b = x + 1.0 - a, c = 1.0 / CF_TINY, d = 1.0 / b, h = d;
  for (int i = 1; i <= CF_MAXIT; ++i) {
    const double an = -i * (i - a);
    b += 2.0;
    d = an * d + b;
    if (fabs(d) < CF_TINY) d = CF_TINY;
    c = b + an / c;
    if (fabs(c) < CF_TINY) c = CF_TINY;
    d = 1.0 / d;
    const double del = d * c;
    h *= del;
    if (fabs(del - 1.0) < CF_EPS) break;
  }
  return exp(lpre) * h;
}

double gp_ftail(int df1, int df2, double F)
{
  /* below 1e-6 (or without degrees of freedom) the reference answers 1 */
  if (F < 0.000001 || df1 < 1 || df2 < 1) return 1.0;
  const double x = (double)df2 / ((double)df2 + (double)df1 * F);
  const double q = gp_betai(0.5 * df2, 0.5 * df1, x);
  /* the reference forms 1 - P(F' <= F): tails below the double spacing at 1 print as 0 */
  double p = 1.0 - q;
  if (p < 0.0) p = 0.0;
  if (p > 1.0) p = 1.0;
  return 1.0 - p;
}

double gp_chitail(int df, double z)
{
  if (df == 1) return erfc(sqrt(0.5 * z));
  if (df == 2) return exp(-0.5 * z);
  if (df <= 0) return 1.0;
  return gp_gammq(0.5 * df, 0.5 * z);
}
