/*
 * gpusmartpca — drop-in for `smartpca -p parfile` on the smartpca hot path, on one GB300.
 *
 * Reads the same parfile keys (readcommands src/eigensrc/smartpca.c:2055-2233) for the
 * options this path supports, the same genotype/SNP/sample files, runs gp_smartpca_run and
 * writes the same outputs:
 *   evaloutname      all eigenvalues, "%12.6f\n" (smartpca.c:1425-1431)
 *   evecoutname      "#eigvals:" header "%20s " + K x "%9.3f " (:1433-1437), then per
 *                    printed sample "%20s " ID, K x "%10.4f  " (hiprecision "%12.6f  ") and
 *                    "%15s\n" population (:1570-1591); fastmode as printevecs (:3837-3871)
 *   outlieroutname   "REMOVED outlier %s iter %d evec %d sigmage %.3f pop: %s\n" (:1255-1257)
 * One extra key selects the Gram precision: gpuprecision: FP64 (default, the drop-in),
 * SPLIT_BF16, SPLIT_BF16X4 or SPLIT_FP16 (include/gpupca.h).  Keys of the reference's other analyses (Fst, ANOVA, shrinkage, LD regression,
 * GRM dump) are accepted and ignored with a note.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "../../include/gpupca.h"
#include "../../include/gpupca_run.h"
#include "gp_io.h"
#include "gp_stats.h"

static void usage(void) { fprintf(stderr, "usage: gpusmartpca -p parfile\n"); }

/* get3 (src/admutils.c:1224-1237): the first character of a name and a blank */
static const char *get3(const char *s)
{
  static char x[4];
  x[0] = s[0] ? s[0] : ' ';
  x[1] = ' ';
  x[2] = 0;
  return x;
}

/* printmatz5 / printmatz10 (src/admutils.c:1185-1221): lrint(scale * value) per entry */
static void printmatz(const double *w, char **eg, int n, int wide)
{
  const double scale = wide ? 1000000.0 : 1000.0;
  printf(" %5s", "   ");
  for (int i = 0; i < n; ++i) printf(wide ? " %10s" : " %5s", get3(eg[i]));
  printf("\n");
  for (int i = 0; i < n; ++i) {
    printf("%5s", get3(eg[i]));
    for (int j = 0; j < n; ++j) printf(wide ? " %10d" : " %5d", (int)lrint(scale * w[i * n + j]));
    printf("\n");
  }
}

static double clipd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

/* centred values and population means (calcmean src/qpsubs.c:430-458): w0 = vec - mean,
 * wmean[k] = sum of w0 over population k / (size + 1e-12); returns the sizes + 1e-12 */
static void pop_means(const double *vec, int len, const int32_t *xt, int numeg, double *w0,
                      double *wmean, double *psz)
{
  double s = 0.0;
  for (int i = 0; i < len; ++i) s += vec[i];
  const double y1 = s / (double)len;
  for (int i = 0; i < len; ++i) w0[i] = vec[i] + -y1;
  for (int k = 0; k < numeg; ++k) wmean[k] = psz[k] = 0.0;
  for (int i = 0; i < len; ++i) {
    psz[xt[i]] += 1.0;
    wmean[xt[i]] += w0[i];
  }
  for (int k = 0; k < numeg; ++k) {
    psz[k] = psz[k] + 1.0e-12;
    wmean[k] = wmean[k] / psz[k];
  }
}

/* anova (smartpca.c:2419-2476): F test of the population means, its upper tail */
static double anova_f(const double *vec, int len, const int32_t *xt, int numeg, double *w0,
                      double *wm, double *psz)
{
  if (numeg >= len) {
    printf("*** warning: bad anova popsizes too small\n");
    return 0.0;
  }
  pop_means(vec, len, xt, numeg, w0, wm, psz);
  double top = 0.0, bot = 0.0;
  for (int k = 0; k < numeg; ++k) top += (wm[k] * wm[k]) * psz[k];
  for (int i = 0; i < len; ++i) {
    const double d = w0[i] - wm[xt[i]];
    bot += d * d;
  }
  bot = bot / (double)(len - numeg);
  bot *= (double)(numeg - 1);
  return gp_ftail(numeg - 1, len - numeg, top / bot);
}

/* anova1 (smartpca.c:2479-2515): log likelihood ratio 0.5 n log(var0 / var1) */
static double anova_ll(const double *vec, int len, const int32_t *xt, int numeg, double *w0,
                       double *wm, double *psz)
{
  pop_means(vec, len, xt, numeg, w0, wm, psz);
  double y1 = 0.0, y2 = 0.0;
  for (int i = 0; i < len; ++i) y1 += w0[i] * w0[i];
  for (int i = 0; i < len; ++i) {
    const double d = w0[i] - wm[xt[i]];
    y2 += d * d;
  }
  y1 = y1 / (double)len;
  y2 = y2 / (double)len;
  return 0.5 * ((double)len) * log(y1 / y2);
}

/* publishit (smartpca.c:2518-2571) without chisqmode: name with blanks as underscores, the
 * p-value, *** below 0.001 and +++ below 1e-6 */
static void publish(const char *sss, double tail, int *ncall)
{
  char ss2[512];
  snprintf(ss2, sizeof ss2, "%s", sss);
  for (char *q = ss2; *q; ++q)
    if (*q == ' ') *q = '_';
  if ((*ncall)++ == 0) {
    printf("## Anova statistics for population differences along each eigenvector:\n");
    printf("%40s %12s\n", "", "p-value");
  }
  printf("%40s ", ss2);
  printf(" %12.6g", tail);
  printf(" %s", tail < 1.0e-6 ? "+++" : (tail < 0.001 ? "***" : ""));
  printf("\n");
}

/*
 * The ANOVA tail of smartpca's log (dottest smartpca.c:2316-2417 per eigenvector, then the
 * popdifference table :1977-1993): population means of each eigenvector (sorted), the F-test
 * p-value overall and per population pair, and per pair the chi-square of the summed
 * likelihood ratios over the eigenvectors with its upper tail.  Eigenvector signs are the
 * eigensolver's, so the means (and minv/maxv) may come out negated against the reference.
 */
static void anova_tail(const gp_run_result *r, char **eg, int numeg, const int32_t *xt,
                       const int32_t *psize)
{
  const int n = r->nrows, K = r->numeigs;
  double *w0 = (double *)malloc(sizeof(double) * (size_t)(n + numeg + 2));
  double *wv = (double *)malloc(sizeof(double) * (size_t)(n + 2));
  int32_t *xt2 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 2));
  double *wm = (double *)malloc(sizeof(double) * (size_t)numeg), *psz = (double *)malloc(sizeof(double) * (size_t)numeg);
  double *chitot = (double *)calloc((size_t)numeg * numeg, sizeof(double));
  int *ord = (int *)malloc(sizeof(int) * (size_t)numeg);
  int ncall = 0;
  for (int j = 0; j < K; ++j) {
    const double *vec = r->evecs + (size_t)j * n;
    char sss[64];
    snprintf(sss, sizeof sss, "eigenvector %d", j + 1);
    pop_means(vec, n, xt, numeg, w0, wm, psz);
    /* sortit: ascending, ties in index order */
    for (int k = 0; k < numeg; ++k) ord[k] = k;
    for (int a = 1; a < numeg; ++a) {
      const int v = ord[a];
      int b = a - 1;
      while (b >= 0 && wm[ord[b]] > wm[v]) {
        ord[b + 1] = ord[b];
        --b;
      }
      ord[b + 1] = v;
    }
    printf("%s:means\n", sss);
    for (int i = 0; i < numeg; ++i) {
      printf("%20s ", eg[ord[i]]);
      printf(" %9.3f\n", wm[ord[i]]);
    }
    int imax = 0, imin = 0;
    for (int k = 1; k < numeg; ++k) {
      if (wm[k] > wm[imax]) imax = k;
      if (wm[k] < wm[imin]) imin = k;
    }
    const double wmin = wm[imin], wmax = wm[imax];
    const double ans = anova_f(vec, n, xt, numeg, w0, wm, psz);
    if (numeg > 2) {
      char s2[128];
      snprintf(s2, sizeof s2, "%s %s ", sss, "overall");
      publish(s2, ans, &ncall);
      printf(" %20s minv: %9.3f %20s maxv: %9.3f\n", eg[imin], wmin, eg[imax], wmax);
    }
    for (int k1 = 0; k1 < numeg; ++k1) {
      for (int k2 = k1 + 1; k2 < numeg; ++k2) {
        int m = 0, x1 = 0, x2 = 0;
        for (int i = 0; i < n; ++i) {
          if (xt[i] == k1) {
            wv[m] = vec[i];
            xt2[m++] = 0;
            ++x1;
          }
          if (xt[i] == k2) {
            wv[m] = vec[i];
            xt2[m++] = 1;
            ++x2;
          }
        }
        if (x1 <= 1 || x2 <= 1) continue;
        chitot[k1 * numeg + k2] += 2.0 * anova_ll(wv, m, xt2, 2, w0, wm, psz);
        const double ansx = anova_f(wv, m, xt2, 2, w0, wm, psz);
        char s2[256];
        snprintf(s2, sizeof s2, "%s %s %s ", sss, eg[k1], eg[k2]);
        publish(s2, ansx, &ncall);
      }
    }
  }
  printf("\n## Statistical significance of differences beween populations:\n");
  printf("                                pop1                  pop2      chisq          p-value   |pop1|   |pop2|\n");
  for (int k1 = 0; k1 < numeg; ++k1) {
    for (int k2 = k1 + 1; k2 < numeg; ++k2) {
      const double ychi = chitot[k1 * numeg + k2];
      printf("popdifference:  %20s  %20s  %12.3f  %12.6g", eg[k1], eg[k2], ychi,
             gp_chitail(K, ychi));
      printf("   %5d", psize[k1]);
      printf("   %5d", psize[k2]);
      printf("\n");
    }
  }
  printf("\n");
  free(w0);
  free(wv);
  free(xt2);
  free(wm);
  free(psz);
  free(chitot);
  free(ord);
}

/*
 * The population summary and Fst section of smartpca's log after the PCA
 * (src/eigensrc/smartpca.c:1784-1961): population sizes over the rows of the last pass, the
 * block count, the Fst matrix and its jackknife standard errors (gp_fst), and the optional
 * phylip / mega / fstdetails files.
 */
/* the number of populations of the eglist (smartpca.c:774-784): the poplist's entries, else
 * the distinct populations of the samples not ignored */
static int count_eglist(const gp_indlist *inds, const char *poplistname, int32_t N)
{
  int numeg = 0;
  if (poplistname) {
    FILE *pl = fopen(poplistname, "r");
    char line[1024];
    while (pl && fgets(line, sizeof line, pl)) {
      char w[256];
      if (sscanf(line, "%255s", w) != 1 || w[0] == '#') continue;
      ++numeg;
    }
    if (pl) fclose(pl);
    return numeg;
  }
  const char **eg = (const char **)malloc(sizeof(char *) * (size_t)(N + 1));
  if (!eg) return 0;
  for (int32_t k = 0; k < N; ++k) {
    if (inds->ignore[k]) continue;
    int found = 0;
    for (int e = 0; e < numeg && !found; ++e) found = strcmp(eg[e], inds->pop[k]) == 0;
    if (!found) eg[numeg++] = inds->pop[k];
  }
  free(eg);
  return numeg;
}

static int fst_tail(gp_ctx *ctx, const gp_parfile *pf, const gp_snplist *snps,
                    const gp_indlist *inds, const gp_run_result *r, const char *poplistname,
                    int64_t M, int32_t N)
{
  const char *phylipname = NULL, *fstdetailsname = NULL, *megaoutname = NULL;
  int32_t fstverbose = 0, fsthiprec = 0, fstz = 0, t = 0;
  double blgsize = 0.05;
  gp_par_str(pf, "phylipname:", &phylipname);
  gp_par_str(pf, "phylipoutname:", &phylipname);
  gp_par_str(pf, "fstdetailsname:", &fstdetailsname);
  gp_par_str(pf, "megaoutname:", &megaoutname);
  gp_par_int(pf, "fstverbose:", &fstverbose);
  gp_par_int(pf, "fsthiprecision:", &fsthiprec);
  gp_par_int(pf, "fstz:", &fstz);
  gp_par_dbl(pf, "blgsize:", &blgsize);
  if (gp_par_int(pf, "inbreed:", &t) && t) {
    printf("inbreed: YES is not supported by this path; no Fst section\n");
    return 0;
  }
  /* eglist: the poplist order, else the order of first appearance (makeeglist) */
  char **eg = (char **)malloc(sizeof(char *) * (size_t)(N + 4096));
  int numeg = 0;
  if (poplistname) {
    FILE *pl = fopen(poplistname, "r");
    char line[1024];
    while (pl && fgets(line, sizeof line, pl)) {
      char w[256];
      if (sscanf(line, "%255s", w) != 1 || w[0] == '#') continue;
      eg[numeg++] = strdup(w);
    }
    if (pl) fclose(pl);
  } else {
    for (int32_t k = 0; k < N; ++k) {
      if (inds->ignore[k]) continue;
      int found = 0;
      for (int e = 0; e < numeg && !found; ++e) found = strcmp(eg[e], inds->pop[k]) == 0;
      if (!found) eg[numeg++] = strdup(inds->pop[k]);
    }
  }
  if (numeg < 1) return 0;
  int32_t *xt = (int32_t *)malloc(sizeof(int32_t) * (size_t)r->nrows);
  int32_t *psize = (int32_t *)calloc((size_t)numeg, sizeof(int32_t));
  for (int32_t i = 0; i < r->nrows; ++i) {
    xt[i] = -1;
    for (int e = 0; e < numeg; ++e)
      if (strcmp(eg[e], inds->pop[r->xindex[i]]) == 0) {
        xt[i] = e;
        break;
      }
    if (xt[i] >= 0) ++psize[xt[i]];
  }
  for (int e = 0; e < numeg; ++e) {
    printf("population: %3d %20s %4d", e, eg[e], psize[e]);
    if (psize[e] == 0) printf(" ***");
    printf("\n");
  }
  /* jackknife blocks over the SNPs still in use (numblocks / setblocks) */
  int32_t *chrom = (int32_t *)malloc(sizeof(int32_t) * (size_t)M);
  double *gpos = (double *)malloc(sizeof(double) * (size_t)M);
  uint8_t *ign = (uint8_t *)malloc((size_t)M);
  int32_t *tag = (int32_t *)malloc(sizeof(int32_t) * (size_t)M);
  for (int64_t i = 0; i < M; ++i) {
    chrom[i] = snps->chrom[snps->order[i]];
    gpos[i] = snps->gpos[snps->order[i]];
    ign[i] = r->snp_state[i] != 0;
  }
  const int32_t nblocks = gp_set_blocks(chrom, gpos, ign, M, blgsize, tag);
  printf("number of blocks for block jackknife: %d\n", nblocks);
  if (nblocks == 1) printf("number of blocks 1: no standard error\n");
  const size_t EE = (size_t)numeg * numeg;
  double *fmean = (double *)calloc(EE, sizeof(double)), *fans = (double *)calloc(EE, sizeof(double));
  double *fsd = (double *)calloc(EE, sizeof(double));
  int32_t *fnum = (int32_t *)calloc(EE, sizeof(int32_t));
  if (nblocks >= 1) {
    int rc = gp_fst(ctx, xt, numeg, tag, nblocks, fmean, fans, fsd, fnum);
    if (rc) return rc;
  }
  if (megaoutname) {
    /* printmega (smartpca.c:4785-4812) */
    FILE *f = fopen(megaoutname, "w");
    if (f) {
      fprintf(f, "#mega\n");
      fprintf(f, "!TITLE distance for %d samples ;", numeg);
      fprintf(f, "\n\n");
      for (int i = 0; i < numeg; i++) fprintf(f, "#%s\n", eg[i]);
      fprintf(f, "\n\n");
      for (int i = 0; i < numeg; i++) {
        for (int j = 0; j < i; j++) {
          double y = fans[i * numeg + j];
          fprintf(f, "  %9.6f", y > 0 ? y : 0);
        }
        fprintf(f, "\n");
      }
      fclose(f);
    }
  }
  if ((phylipname == NULL && numeg > 10) || fstverbose) {
    printf("## Fst statistics between populations:         fst       std error      Z\n");
    for (int k1 = 0; k1 < numeg; ++k1) {
      for (int k2 = k1 + 1; k2 < numeg; ++k2) {
        const double z = fans[k1 * numeg + k2] / (fsd[k1 * numeg + k2] + 1.0e-10);
        if (!fsthiprec)
          printf(" %20s %20s %9.3f %10.4f", eg[k1], eg[k2], fans[k1 * numeg + k2],
                 fsd[k1 * numeg + k2]);
        else
          printf(" %20s %20s %12.6f %12.6f", eg[k1], eg[k2], fans[k1 * numeg + k2],
                 fsd[k1 * numeg + k2]);
        printf("  %9.3f ", z);
        printf(" %12d", fnum[k1 * numeg + k2]);
        printf("\n");
      }
    }
    printf("\n");
  }
  printf("## end of Fst statistics between populations\n");
  if (fstdetailsname) {
    FILE *f = fopen(fstdetailsname, "w");
    if (f) {
      fprintf(f, "## Fst statistics between populations:     fst     fstjack       std error      Z    snpnumber\n");
      for (int k1 = 0; k1 < numeg; ++k1)
        for (int k2 = k1 + 1; k2 < numeg; ++k2) {
          const int k = k1 * numeg + k2;
          if (!fsthiprec)
            fprintf(f, "F_st %20s %20s %12.6f %12.6f %12.6f", eg[k1], eg[k2], fmean[k], fans[k],
                    fsd[k]);
          else
            fprintf(f, "F_st %20s %20s %15.9f %15.9f %15.9f", eg[k1], eg[k2], fmean[k], fans[k],
                    fsd[k]);
          fprintf(f, " %9.3f", fans[k] / (fsd[k] + 1.0e-10));
          fprintf(f, " %6d", fnum[k]);
          fprintf(f, "\n");
        }
      fclose(f);
    }
  }
  if (fstz) {
    double *zz = (double *)malloc(sizeof(double) * EE);
    memcpy(zz, fans, sizeof(double) * EE);
    for (int k1 = 0; k1 < numeg; ++k1)
      for (int k2 = k1 + 1; k2 < numeg; ++k2)
        zz[k2 * numeg + k1] =
            clipd(fans[k1 * numeg + k2] / (fsd[k1 * numeg + k2] + 1.0e-10), -9.999999, 9.999999);
    printf("\n");
    printf(fsthiprec ? "Fst: Z/F *1000000 [clipped to -10,10]\n" : "Fst: Z/F *1000 [clipped to -10,10]\n");
    printmatz(zz, eg, numeg, fsthiprec);
    free(zz);
  }
  printf("\n");
  if (phylipname) {
    FILE *f = fopen(phylipname, "w");
    if (f) {
      fprintf(f, "%6d\n", numeg);
      for (int k1 = 0; k1 < numeg; ++k1) {
        char sss[11];
        snprintf(sss, sizeof sss, "%.10s", eg[k1]);
        fprintf(f, "%10s", sss);
        for (int k2 = 0; k2 < numeg; ++k2)
          fprintf(f, "%6.3f", 0.5 * (fans[k1 * numeg + k2] + fans[k2 * numeg + k1]));
        fprintf(f, "\n");
      }
      fclose(f);
    }
  }
  if (numeg <= 10) {
    printf(fsthiprec ? "fst *1000000:" : "fst *1000:");
    printf("\n");
    printmatz(fans, eg, numeg, fsthiprec);
    printf("\n");
  }
  printf("std. err.  * 1000000:\n");
  for (size_t i = 0; i < EE; ++i) fsd[i] *= 1000.0;
  printmatz(fsd, eg, numeg, 0);
  printf("\n");
  anova_tail(r, eg, numeg, xt, psize);
  free(fmean);
  free(fans);
  free(fsd);
  free(fnum);
  free(chrom);
  free(gpos);
  free(ign);
  free(tag);
  free(xt);
  free(psize);
  return 0;
}

static int in_list(const char *pop, char **list, int n)
{
  for (int i = 0; i < n; ++i)
    if (strcmp(pop, list[i]) == 0) return 1;
  return 0;
}

/* kurtosis (src/admutils.c:995-1017): the mean fourth power of the standardised values,
 * every sum in index order */
static double kurtosis_of(const double *a, int64_t n)
{
  double y1 = 0.0, y2 = 0.0, y4 = 0.0;
  for (int64_t i = 0; i < n; ++i) y1 += a[i];
  y1 = y1 / (double)n;
  for (int64_t i = 0; i < n; ++i) {
    const double w = a[i] + -y1;
    y2 += w * w;
  }
  y2 = y2 / (double)n;
  const double sc = 1.0 / sqrt(y2);
  for (int64_t i = 0; i < n; ++i) {
    double w = (a[i] + -y1) * sc;
    w = w * w;
    y4 += w * w;
  }
  return y4 / (double)n;
}

/*
 * The mpstats line and the Tracy-Widom section of the log (smartpca.c:1306-1367; mpestimate
 * :4532-4560): over the m eigenvalues of the last pass above 1e-6 (numgtz), the quartile line
 * when m >= 10, then per eigenvalue its difference to the previous one, the statistic, the TW1
 * tail and the effective number of markers (NA where fewer than nostatslim eigenvalues
 * remain).  The statistics come from gp_twstats / gp_mpstats.
 */
static int tw_lines(const gp_run_result *r, int nostatslim)
{
  const int32_t n = r->nrows;
  int32_t m = 0;
  for (int32_t i = 0; i < n; ++i)
    if (r->evals[i] > 0.000001) ++m;
  if (m == 0) return 0;
  double q[4];
  if (gp_mpstats(r->evals, m, q) == GP_OK)
    printf("mpstats: %9.3f%9.3f%9.3f%12.6f\n", q[0], q[1], q[2], q[3]);
  double *tw = (double *)malloc(sizeof(double) * 3 * (size_t)m);
  if (!tw) return -1;
  double *pv = tw + m, *zn = pv + m;
  if (gp_twstats(r->evals, m, n, -1.0, nostatslim, tw, pv, zn) != GP_OK) {
    free(tw);
    return -1;
  }
  printf("\n## Tracy-Widom statistics: rows: %d  cols: %d\n", n, r->ncols);
  printf("%4s  %12s", "#N", "eigenvalue");
  printf("%12s", "difference");
  printf(" %9s %12s", "twstat", "p-value");
  printf(" %9s", "effect. n");
  printf("\n");
  for (int32_t i = 0; i < m; ++i) {
    printf("%4d  %12.6f", i + 1, r->evals[i]);
    if (i == 0)
      printf("%12s", "NA");
    else
      printf("%12.6f", r->evals[i] - r->evals[i - 1]);
    if (pv[i] >= 0.0)
      printf(" %9.3f %12.6g", tw[i], pv[i]);
    else
      printf(" %9s %12s", "NA", "NA");
    if (zn[i] > 0.0)
      printf(" %9.3f", zn[i]);
    else
      printf(" %9s", "NA");
    printf("\n");
  }
  free(tw);
  return 0;
}

/*
 * The kurtosis lines of the log (smartpca.c:1496-1501, :1541-1546): per eigenvector the
 * kurtosis of its SNP weights over the last pass's columns (zeros for the SNPs that pass
 * dropped) and of 10 x its entries over the rows.
 */
static int kurtosis_lines(const gp_run_result *r, int64_t M)
{
  const int32_t K = r->numeigs, n = r->nrows, nc = r->ncols;
  if (!r->ffvecs || !r->snp_lastpass || K < 1) return 0;
  double *col = (double *)malloc(sizeof(double) * (size_t)(nc > n ? nc : n) + 8);
  if (!col) return -1;
  printf("%12s %4s %9s %9s\n", "kurtosis", "", "snps", "indivs");
  for (int32_t j = 0; j < K; ++j) {
    int64_t m = 0;
    for (int64_t s = 0; s < M; ++s)
      if (r->snp_lastpass[s]) col[m++] = r->ffvecs[(size_t)j * M + s];
    const double ks = kurtosis_of(col, m);
    for (int32_t i = 0; i < n; ++i) col[i] = r->evecs[(size_t)j * n + i] * 10.0;
    const double ki = kurtosis_of(col, n);
    printf("%12s %4d %9.3f %9.3f\n", "eigenvector", j + 1, ks, ki);
  }
  free(col);
  return 0;
}

/*
 * writesnpeigs (src/eigensrc/smartpca.c:3038-3106): each eigenvector's SNP weights scaled to
 * mean square 1 over the last pass's columns (sum of squares in column order, then
 * sqrt(ncols / sum)), the "eigbestsnp" log lines (per eigenvector the 10 largest |weight| of
 * the SNPs still in use, the first of equal values first, none when ncols <= 10), and the
 * snpweightoutname file when a path is given: per SNP in use its ID, chromosome, physical
 * position and weights.
 */
static int snp_weights_tail(const char *path, gp_run_result *r, const gp_snplist *snps,
                            int64_t M, int hiprec)
{
  const int32_t K = r->numeigs, ncols = r->ncols;
  double *f = r->ffvecs;
  if (!f || K < 1) return 0;
  for (int32_t j = 0; j < K; ++j) {
    double *w = f + (size_t)j * M, y = 0.0;
    for (int64_t s = 0; s < M; ++s)
      if (r->snp_state[s] == 0) y += w[s] * w[s];
    double ysc = (double)ncols / y;
    ysc = sqrt(ysc);
    for (int64_t s = 0; s < M; ++s)
      if (r->snp_state[s] == 0) w[s] = w[s] * ysc;
  }
  double *sc = (double *)malloc(sizeof(double) * (size_t)(M > 0 ? M : 1));
  if (!sc) return -1;
  for (int32_t j = 0; j < K; ++j) {
    const double *w = f + (size_t)j * M;
    for (int64_t s = 0; s < M; ++s) sc[s] = r->snp_state[s] == 0 ? fabs(w[s]) : -99999.0;
    for (int k = 0; k < 10; ++k) {
      if (ncols <= 10) break;
      int64_t best = -1;
      for (int64_t s = 0; s < M; ++s)
        if (r->snp_state[s] == 0 && (best < 0 || sc[s] > sc[best])) best = s;
      if (best < 0 || sc[best] < 0) break;
      const int64_t row = snps->order[best];
      printf("eigbestsnp %4d %20s %2d %12d %9.3f\n", j + 1, snps->id[row], snps->chrom[row],
             (int)lrint(snps->ppos[row]), sc[best]);
      sc[best] = -1.0;
    }
  }
  free(sc);
  if (!path) return 0;
  FILE *fo = fopen(path, "w");
  if (!fo) {
    fprintf(stderr, "cannot write %s\n", path);
    return -1;
  }
  for (int64_t s = 0; s < M; ++s) {
    if (r->snp_state[s] != 0) continue;
    const int64_t row = snps->order[s];
    fprintf(fo, "%20s", snps->id[row]);
    fprintf(fo, " %2d", snps->chrom[row]);
    fprintf(fo, " %12d", (int)lrint(snps->ppos[row]));
    for (int32_t j = 0; j < K; ++j) {
      if (hiprec) fprintf(fo, " %12.6f", f[(size_t)j * M + s]);
      else fprintf(fo, " %9.3f", f[(size_t)j * M + s]);
    }
    fprintf(fo, "\n");
  }
  fclose(fo);
  return 0;
}

int main(int argc, char **argv)
{
  const char *parname = NULL;
  int c;
  while ((c = getopt(argc, argv, "p:vV")) != -1) {
    if (c == 'p') parname = optarg;
    else if (c == 'v') printf("version: gpusmartpca %d\n", gp_version());
  }
  if (!parname) {
    usage();
    return 1;
  }
  gp_parfile pf;
  if (gp_par_read(parname, &pf) != 0) {
    fprintf(stderr, "can't open %s\n", parname);
    return 1;
  }
  printf("parameter file: %s\n", parname);
  printf("### THE INPUT PARAMETERS\n##PARAMETER NAME: VALUE\n");
  for (int k = 0; k < pf.n; ++k) printf("%s %s\n", pf.key[k], pf.val[k]);

  gp_smartpca_opts o;
  gp_smartpca_defaults(&o);
  const char *genotypename = NULL, *snpname = NULL, *indivname = NULL, *evecout = NULL,
             *evalout = NULL, *outlierout = NULL, *poplistname = NULL, *prec = NULL,
             *grmout = NULL, *snpwtout = NULL;
  int32_t hiprec = 0, familynames = 1, hashcheck = 1, t = 0, xdata = -1, seed = 0,
          grmbinary = 0, nostatslim = 10;
  gp_par_str(&pf, "genotypename:", &genotypename);
  gp_par_str(&pf, "snpname:", &snpname);
  gp_par_str(&pf, "indivname:", &indivname);
  gp_par_str(&pf, "poplistname:", &poplistname);
  gp_par_str(&pf, "output:", &evecout);
  gp_par_str(&pf, "outputvecs:", &evecout);
  gp_par_str(&pf, "evecoutname:", &evecout);
  gp_par_str(&pf, "outputvals:", &evalout);
  gp_par_str(&pf, "evaloutname:", &evalout);
  gp_par_str(&pf, "outliername:", &outlierout);
  gp_par_str(&pf, "outlieroutname:", &outlierout);
  gp_par_str(&pf, "gpuprecision:", &prec);
  gp_par_str(&pf, "grmoutname:", &grmout);
  gp_par_str(&pf, "snpeigname:", &snpwtout);
  gp_par_str(&pf, "snpweightoutname:", &snpwtout);
  gp_par_int(&pf, "grmbinary:", &grmbinary);
  gp_par_int(&pf, "numeigs:", &o.numeigs);
  gp_par_int(&pf, "numoutevec:", &o.numeigs);
  gp_par_int(&pf, "nostatslim:", &nostatslim);
  gp_par_int(&pf, "fancynorm:", &o.fancynorm);
  gp_par_int(&pf, "usenorm:", &o.fancynorm);
  gp_par_int(&pf, "altnormstyle:", &o.altnormstyle);
  gp_par_int(&pf, "popgenmode:", &o.altnormstyle);
  gp_par_int(&pf, "hashcheck:", &hashcheck);
  gp_par_int(&pf, "noxdata:", &o.noxdata);
  if (gp_par_int(&pf, "xdata:", &xdata) && xdata >= 0) o.noxdata = 1 - xdata;
  if (gp_par_int(&pf, "seed:", &seed)) o.seed = seed;
  gp_par_int(&pf, "fastmode:", &o.fastmode);
  gp_par_int(&pf, "fastdim:", &o.fastdim);
  gp_par_int(&pf, "fastiter:", &o.fastiter);
  gp_par_int(&pf, "regmode:", &o.lsqproject);
  gp_par_int(&pf, "lsqproject:", &o.lsqproject);
  gp_par_int(&pf, "minallelecnt:", &o.minallelecnt);
  gp_par_int(&pf, "maxmissing:", &o.maxmissing);
  gp_par_int(&pf, "hiprecision:", &hiprec);
  gp_par_int(&pf, "hiprec:", &hiprec);
  gp_par_int(&pf, "familynames:", &familynames);
  gp_par_int(&pf, "numoutliter:", &o.numoutliter);
  gp_par_int(&pf, "numoutlieriter:", &o.numoutliter);
  gp_par_int(&pf, "numoutleigs", &o.numoutleigs);
  gp_par_int(&pf, "numoutlierevec:", &o.numoutleigs);
  gp_par_dbl(&pf, "outlthresh:", &o.outlthresh);
  gp_par_dbl(&pf, "outliersigmathresh:", &o.outlthresh);
  gp_par_int(&pf, "outliermode:", &o.outliermode);
  gp_par_int(&pf, "numchrom:", &o.numchrom);
  gp_par_int(&pf, "missingmode:", &o.missingmode);
  gp_par_int(&pf, "usepopsformissing:", &o.usepopsformissing);
  if (gp_par_int(&pf, "ldregress:", &t) && t > 0) {
    fprintf(stderr, "ldregress is not supported by this path\n");
    return 1;
  }
  if (prec) {
    if (strcmp(prec, "FP64") == 0) o.precision = GP_PREC_FP64;
    else if (strcmp(prec, "SPLIT_BF16") == 0) o.precision = GP_PREC_SPLIT_BF16;
    else if (strcmp(prec, "SPLIT_BF16X4") == 0) o.precision = GP_PREC_SPLIT_BF16X4;
    else if (strcmp(prec, "SPLIT_FP16") == 0) o.precision = GP_PREC_SPLIT_FP16;
    else {
      fprintf(stderr, "gpuprecision: %s is not FP64, SPLIT_BF16, SPLIT_BF16X4 or SPLIT_FP16\n", prec);
      return 1;
    }
  }
  if (o.fastmode) {
    if (o.fastiter < 0) o.fastiter = o.numeigs;
    if (o.fastdim < 0) o.fastdim = 2 * o.numeigs;
    /* rngmode (smartpca.c:679-684): seed 0 draws a seed from the process id, user id and
     * clock, as seednum does, and the seed is logged */
    if (o.seed == 0)
      o.seed = (int64_t)(((long)getpid() + (long)getuid()) << 15) ^ (int64_t)time(NULL);
    printf("seed: %ld\n", (long)o.seed);
  }
  if (!genotypename || !snpname || !indivname) {
    fprintf(stderr, "genotypename, snpname and indivname are required\n");
    return 1;
  }

  char err[512];
  gp_snplist snps;
  gp_indlist inds;
  if (gp_read_snps(snpname, o.numchrom, &snps, err, sizeof err) ||
      gp_read_inds(indivname, familynames, &inds, err, sizeof err)) {
    fprintf(stderr, "%s\n", err);
    return 1;
  }
  uint8_t *records = NULL;
  int64_t rb = 0;
  int32_t code = 0;
  if (gp_read_genotypes(genotypename, &snps, &inds, hashcheck, &records, &rb, &code, err,
                        sizeof err)) {
    fprintf(stderr, "%s\n", err);
    return 1;
  }
  const int64_t M = snps.n;
  const int32_t N = inds.n;
  int32_t *chrom = (int32_t *)malloc(sizeof(int32_t) * (size_t)M);
  for (int64_t i = 0; i < M; ++i) chrom[i] = snps.chrom[snps.order[i]];
  uint8_t *aff = NULL, *male = (uint8_t *)malloc((size_t)N);
  for (int32_t k = 0; k < N; ++k) male[k] = inds.gender[k] == 'M';
  if (poplistname) {
    FILE *pl = fopen(poplistname, "r");
    if (!pl) {
      fprintf(stderr, "cannot open %s\n", poplistname);
      return 1;
    }
    char line[1024], *names[4096];
    int nn = 0;
    while (fgets(line, sizeof line, pl) && nn < 4096) {
      char w[256];
      if (sscanf(line, "%255s", w) != 1 || w[0] == '#') continue;
      names[nn++] = strdup(w);
    }
    fclose(pl);
    aff = (uint8_t *)calloc((size_t)N, 1);
    for (int32_t k = 0; k < N; ++k) aff[k] = (uint8_t)in_list(inds.pop[k], names, nn);
  }

  /* usepopsformissing: each sample's index in the population list (xtypes, smartpca.c:
   * 928-943): the poplist order, else the order of first appearance among the samples not
   * ignored (makeeglist); -1 when the population is not listed */
  int32_t *ind_pop = NULL;
  if (o.usepopsformissing) {
    if (o.fastmode) {
      fprintf(stderr, "usepopsformissing with fastmode is not supported by this path\n");
      return 1;
    }
    char **eg = (char **)malloc(sizeof(char *) * (size_t)(N + 4096));
    int numeg = 0;
    if (poplistname) {
      FILE *pl = fopen(poplistname, "r");
      char line[1024];
      while (pl && fgets(line, sizeof line, pl) && numeg < N + 4096) {
        char w[256];
        if (sscanf(line, "%255s", w) != 1 || w[0] == '#') continue;
        eg[numeg++] = strdup(w);
      }
      if (pl) fclose(pl);
    } else {
      for (int32_t k = 0; k < N; ++k) {
        if (inds.ignore[k]) continue;
        int found = 0;
        for (int e = 0; e < numeg && !found; ++e) found = strcmp(eg[e], inds.pop[k]) == 0;
        if (!found) eg[numeg++] = strdup(inds.pop[k]);
      }
    }
    ind_pop = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    for (int32_t k = 0; k < N; ++k) {
      ind_pop[k] = -1;
      for (int e = 0; e < numeg; ++e)
        if (strcmp(eg[e], inds.pop[k]) == 0) {
          ind_pop[k] = e;
          break;
        }
    }
    for (int e = 0; e < numeg; ++e) free(eg[e]);
    free(eg);
  }

  gp_panel p;
  memset(&p, 0, sizeof p);
  p.records = records;
  p.record_bytes = rb;
  p.nsnp = M;
  p.nind = N;
  p.code = code;
  p.snp_chrom = chrom;
  p.ind_ignore = inds.ignore;
  p.ind_affstatus = aff;
  p.ind_male = male;
  p.ind_pop = ind_pop;

  int32_t K = o.numeigs > 0 ? o.numeigs : 1;
  gp_run_result r;
  memset(&r, 0, sizeof r);
  r.xindex = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  r.evals = (double *)calloc((size_t)N, sizeof(double));
  r.evecs = (double *)calloc((size_t)K * N, sizeof(double));
  r.coords = (double *)calloc((size_t)K * N, sizeof(double));
  r.ind_out = (uint8_t *)calloc((size_t)N, 1);
  r.snp_state = (uint8_t *)calloc((size_t)M, 1);
  r.outlier_idx = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  r.outlier_iter = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  r.outlier_vec = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  r.outlier_score = (double *)calloc((size_t)N, sizeof(double));
  if (snpwtout && o.fastmode) {
    fprintf(stderr, "snpweightoutname with fastmode is not supported by this path\n");
    return 1;
  }
  if (!o.fastmode) {
    /* the last pass's SNP weights: the eigbestsnp lines and snpweightoutname */
    r.ffvecs = (double *)calloc((size_t)K * (size_t)M, sizeof(double));
    r.snp_lastpass = (uint8_t *)calloc((size_t)M, 1);
    if (!r.ffvecs || !r.snp_lastpass) {
      fprintf(stderr, "no memory for the SNP weights (%lld SNPs)\n", (long long)M);
      return 1;
    }
  }
  if (grmout && !o.fastmode) {
    r.xtx = (double *)malloc(sizeof(double) * (size_t)N * N);
    if (!r.xtx) {
      fprintf(stderr, "no memory for the GRM (%d samples)\n", N);
      return 1;
    }
  }

  const int32_t npass_max = (o.numoutliter >= 1 ? o.numoutliter + 1 : 1) + 1;
  r.pass_stats = (int32_t *)calloc((size_t)GP_PASS_STATS * npass_max, sizeof(int32_t));
  r.pass_kills = (int32_t *)calloc((size_t)30 * npass_max, sizeof(int32_t));
  if (!r.pass_stats || !r.pass_kills) {
    fprintf(stderr, "no memory for the pass records\n");
    return 1;
  }
  const int numeg_axes = count_eglist(&inds, poplistname, N);

  gp_ctx *ctx = NULL;
  int rc = gp_open(0, &ctx);
  if (rc) {
    fprintf(stderr, "gp_open: %s\n", gp_last_error(NULL));
    return 1;
  }
  rc = gp_smartpca_run(ctx, &o, &p, &r);
  if (rc) {
    fprintf(stderr, "fatalx:\n%s (code %d)\n", gp_last_error(ctx), rc);
    gp_close(ctx);
    return 1;
  }
  /* the reference's progress lines (smartpca.c:715-719, mcio.c:2842/2877 or :3987,
   * smartpca.c:851, :945-946, then per pass :1140-1141, :1223, :1259-1264) */
  printf(o.fancynorm ? "norm used\n\n" : "no norm used\n\n");
  if (o.lsqproject) printf("lsqproject used\n");
  if (code == GP_CODE_BED)
    printf("genotype file processed\n");
  else
    printf("packed geno read OK\nend of inpack\n");
  printf("snps deleted (nodata): %d.  deletesnpoutname: for details", r.nodata);
  printf("number of samples used: %d number of snps used: %d\n", r.nrows0, r.ncols0);
  printf("number of pops for axes: %d\n", numeg_axes);
  FILE *ol = stdout;
  if (outlierout) ol = fopen(outlierout, "w");
  if (o.fastmode) {
    printf("writing eigenvecotrs for  %d samples\n", r.nrows);
  } else {
    /* the reference's kill count starts at 0 once, before the passes (smartpca.c:1074): its
     * "killed in pass" is the running total, and only the first 10 kills of the run are
     * listed */
    int32_t io = 0, nkill = 0;
    for (int32_t pass = 0; pass < r.npasses; ++pass) {
      const int32_t *ps = r.pass_stats + (size_t)GP_PASS_STATS * pass;
      const int32_t *pk = r.pass_kills + (size_t)30 * pass;
      for (int32_t j = 0; j < ps[3] && nkill + j < 10; ++j)
        printf(" snp %20s ignored . allelecnt: %5d  missing: %5d\n", snps.id[pk[3 * j]],
               pk[3 * j + 1], pk[3 * j + 2]);
      nkill += ps[0];
      printf("total number of snps killed in pass: %d  used: %d\n", nkill, ps[1]);
      if (ps[2] < 0) continue;
      for (; io < r.noutliers && r.outlier_iter[io] == pass + 1 && ol; ++io) {
        int32_t k = r.outlier_idx[io];
        fprintf(ol, "REMOVED outlier %s iter %d evec %d sigmage %.3f pop: %s\n", inds.id[k],
                r.outlier_iter[io], r.outlier_vec[io], r.outlier_score[io], inds.pop[k]);
      }
      printf("number of samples after outlier removal: %d\n", ps[2]);
    }
    for (; io < r.noutliers && ol; ++io) { /* none expected: every removal ends a pass */
      int32_t k = r.outlier_idx[io];
      fprintf(ol, "REMOVED outlier %s iter %d evec %d sigmage %.3f pop: %s\n", inds.id[k],
              r.outlier_iter[io], r.outlier_vec[io], r.outlier_score[io], inds.pop[k]);
    }
  }
  if (ol && ol != stdout) fclose(ol);

  if (r.xtx) {
    /* dumpgrm (smartpca.c:1297): the last pass's Gram in xindex order */
    if (gp_write_grm(grmout, grmbinary, r.xtx, r.nrows, r.nused, inds.id, r.xindex, err,
                     (int)sizeof err)) {
      fprintf(stderr, "%s\n", err);
      return 1;
    }
    printf("grm dumped\n");
  }

  int32_t nK = r.numeigs;
  if (evalout && !o.fastmode) {
    FILE *f = fopen(evalout, "w");
    if (!f) {
      fprintf(stderr, "cannot write %s\n", evalout);
      return 1;
    }
    for (int32_t j = 0; j < r.nrows; ++j) fprintf(f, "%12.6f\n", r.evals[j]);
    fclose(f);
  }
  FILE *ef = stdout;
  if (evecout) ef = fopen(evecout, "w");
  if (!ef) {
    fprintf(stderr, "cannot write %s\n", evecout);
    return 1;
  }
  if (nK > 0) {
    fprintf(ef, "%20s ", "#eigvals:");
    for (int32_t j = 0; j < nK; ++j) fprintf(ef, "%9.3f ", r.evals[j]);
    fprintf(ef, "\n");
    for (int32_t k = 0; k < N; ++k) {
      if (!r.ind_out[k]) continue;
      fprintf(ef, "%20s ", inds.id[k]);
      for (int32_t j = 0; j < nK; ++j) {
        double y = r.coords[(size_t)j * N + k];
        if (hiprec) fprintf(ef, "%12.6f  ", y);
        else fprintf(ef, "%10.4f  ", y);
      }
      fprintf(ef, "%15s\n", inds.pop[k]);
    }
  }
  if (ef != stdout) fclose(ef);
  if (!o.fastmode && nK > 0) {
    if (tw_lines(&r, nostatslim < 3 ? 3 : nostatslim)) {
      fprintf(stderr, "no memory for the Tracy-Widom statistics\n");
      gp_close(ctx);
      return 1;
    }
    if (kurtosis_lines(&r, M)) {
      gp_close(ctx);
      return 1;
    }
    if (o.lsqproject) printf("lsqproj called!\n");
    rc = fst_tail(ctx, &pf, &snps, &inds, &r, poplistname, M, N);
    if (rc) {
      fprintf(stderr, "fatalx:\n%s (code %d)\n", gp_last_error(ctx), rc);
      gp_close(ctx);
      return 1;
    }
    if (snp_weights_tail(snpwtout, &r, &snps, M, hiprec)) {
      gp_close(ctx);
      return 1;
    }
  }
  if (o.fastmode) printf("end of smartpca(fastmode)\n");
  printf("## phase seconds: load %.3f filter %.3f gram %.3f eig %.3f outlier %.3f weights %.3f "
         "lsqproj %.3f total %.3f\n",
         r.t_phase[0], r.t_phase[1], r.t_phase[2], r.t_phase[3], r.t_phase[4], r.t_phase[5],
         r.t_phase[6], r.t_phase[7]);
  printf("##end of gpusmartpca\n");
  gp_close(ctx);
  gp_free_snps(&snps);
  gp_free_inds(&inds);
  gp_par_free(&pf);
  free(records);
  return 0;
}
