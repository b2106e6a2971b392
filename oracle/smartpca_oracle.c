/*
 * ORACLE — test infrastructure only.  A CPU restatement of the reference smartpca hot path
 * (EIGENSOFT 8.0.0, DReichLab/EIG) used as the checker by tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference leg.  Nothing in the product links it.
 *
 * Each function names the reference code it restates (paths inside the reference project).
 * Pinned against the reference binary built by oracle/build_ref.sh (golden fixtures in
 * tests/golden/, generated by tests/golden/make_golden.py).
 *
 * Genotypes come in as packedancestrymap records (rlen bytes per SNP, 2-bit MSB first,
 * 3 = missing; src/admutils.c:718-735).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXTHREADS 256

static inline int orc_geno(const uint8_t *rec, int32_t k)
{
  /* rbuff + getgtypes: 3 -> -1 (src/admutils.c:594-606, :718-735) */
  int g = (rec[k >> 2] >> ((3 - (k & 3)) * 2)) & 3;
  return g == 3 ? -1 : g;
}

/* ---- per-SNP counts and normalisation ------------------------------------------------ */

/*
 * getcolxz_binary1 (src/eigensrc/smartpca.c:3219-3301) + fvadjust_binary (:2282-2313):
 * counts over the rows, then the 3-entry table (k - mean)*fancy, xmean = mean*fancy,
 * xfancy = fancy.  Returns nmiss, or -1 when every row is missing (n0 = n1 = -1, table 0).
 */
int orc_snp_column(const uint8_t *rec, const int32_t *xindex, int32_t nrows, int fancynorm,
                   int altnormstyle, int32_t *n0, int32_t *n1, double *tab, double *xmean,
                   double *xfancy)
{
  int c0 = 0, c1 = 0, nmiss = 0;
  for (int32_t j = 0; j < nrows; ++j) {
    int g = orc_geno(rec, xindex[j]);
    if (g < 0) {
      ++nmiss;
      continue;
    }
    c0 += g;
    c1 += 2 - g;
  }
  if (nmiss == nrows) {
    *xmean = 0.0;
    *xfancy = 0.0;
    tab[0] = tab[1] = tab[2] = 0.0;
    *n0 = *n1 = -1;
    return -1;
  }
  double ynum = nrows - nmiss, ysum = c0, ymean = ysum / ynum, yfancy = 1.0, p, y;
  tab[0] = -ymean;
  tab[1] = 1.0 - ymean;
  tab[2] = 2.0 - ymean;
  if (fancynorm) {
    p = 0.5 * ymean;
    if (altnormstyle == 0) p = (ysum + 1.0) / (2.0 * ynum + 2.0);
    y = p * (1.0 - p);
    if (y > 0.0) yfancy = 1.0 / sqrt(y);
  }
  for (int t = 0; t < 3; ++t) tab[t] = tab[t] * yfancy;
  *xmean = ymean * yfancy;
  *xfancy = yfancy;
  *n0 = c0;
  *n1 = c1;
  return nmiss;
}

/*
 * The per-SNP part of the outlier-loop pass (smartpca.c:1116-1144): counts, table, kill
 * rule.  killed[c] = 1 when min(n0,n1) < minallelecnt, nmiss > maxmissing, no data, or
 * min == 0.  tab [4*ncols] (entry 3 = 0 for missing; all 0 when killed).
 */
void orc_pass_columns(const uint8_t *records, int64_t rlen, const int32_t *cols, int32_t ncols,
                      const int32_t *xindex, int32_t nrows, int fancynorm, int altnormstyle,
                      int minallelecnt, int maxmissing, int32_t *n0, int32_t *n1,
                      int32_t *nmiss, uint8_t *killed, double *tab, double *xmean,
                      double *xfancy)
{
  for (int32_t c = 0; c < ncols; ++c) {
    const uint8_t *rec = records + (int64_t)cols[c] * rlen;
    int tt = orc_snp_column(rec, xindex, nrows, fancynorm, altnormstyle, &n0[c], &n1[c],
                            &tab[4 * c], &xmean[c], &xfancy[c]);
    int t = n0[c] < n1[c] ? n0[c] : n1[c];
    nmiss[c] = tt < 0 ? nrows : tt;
    killed[c] = (t < minallelecnt) || (tt > maxmissing) || (tt < 0) || (t == 0);
    if (killed[c]) tab[4 * c] = tab[4 * c + 1] = tab[4 * c + 2] = 0.0;
    tab[4 * c + 3] = 0.0;
  }
}

/* ---- Gram: plain FP64 ------------------------------------------------------------------ */

/* XTX (full n x n) = sum over kept columns of v v^T, v from the tables; plain loops. */
void orc_gram_plain(const uint8_t *records, int64_t rlen, const int32_t *cols, int32_t ncols,
                    const uint8_t *killed, const double *tab, const int32_t *xindex, int32_t n,
                    double *XTX)
{
  double *v = (double *)malloc(sizeof(double) * (size_t)n);
  memset(XTX, 0, sizeof(double) * (size_t)n * n);
  for (int32_t c = 0; c < ncols; ++c) {
    if (killed[c]) continue;
    const uint8_t *rec = records + (int64_t)cols[c] * rlen;
    for (int32_t i = 0; i < n; ++i) {
      int g = orc_geno(rec, xindex[i]);
      v[i] = tab[4 * c + (g < 0 ? 3 : g)];
    }
    for (int32_t i = 0; i < n; ++i) {
      double vi = v[i];
      if (vi == 0.0) continue;
      double *row = XTX + (int64_t)i * n;
      for (int32_t j = 0; j <= i; ++j) row[j] += vi * v[j];
    }
  }
  for (int32_t i = 0; i < n; ++i)
    for (int32_t j = i + 1; j < n; ++j) XTX[(int64_t)i * n + j] = XTX[(int64_t)j * n + i];
  free(v);
}

/* ---- Gram: the reference's partial-sum lookup algorithm, threaded ----------------------- */
/*
 * Restates the PLINK-1.5 partial-sum lookup used by smartpca (getcolxz_binary2
 * smartpca.c:3304-3328, domult_increment_lookup :3426-3495, block_increment_binary
 * :3361-3423, row partition triangle_fill :444-477).  Per block of 20 SNPs every row gets a
 * 64-bit word with a 3-bit field per SNP at bit 3x + x/5 (hom-ref 0 -> 0, het -> 2,
 * hom-alt -> 3) and a missing mask (7 in the field).  For a pair of rows the sum of the two
 * words OR both masks gives a field value 0 (0,0), 2 (0,1), 3 (0,2), 4 (1,1), 5 (1,2),
 * 6 (2,2), 7 (missing); four 16-bit slices of 5 fields index four 32768-entry tables of
 * partial sums of the products t_a t_b.
 */
typedef struct {
  const uint64_t *geno, *mask;
  const double *tabs; /* 4 x 32768 */
  double *xtx;        /* packed lower triangle, row i at i(i+1)/2 */
  int32_t row_lo, row_hi;
} orc_lookup_job;

static void *orc_lookup_worker(void *arg)
{
  orc_lookup_job *jb = (orc_lookup_job *)arg;
  const double *t0 = jb->tabs, *t1 = t0 + 32768, *t2 = t1 + 32768, *t3 = t2 + 32768;
  for (int32_t i = jb->row_lo; i < jb->row_hi; ++i) {
    double *out = jb->xtx + ((int64_t)i * (i + 1)) / 2;
    uint64_t gi = jb->geno[i], mi = jb->mask[i];
    for (int32_t j = 0; j <= i; ++j) {
      uint64_t key = (gi + jb->geno[j]) | mi | jb->mask[j];
      out[j] += t0[(uint16_t)key] + t1[(uint16_t)(key >> 16)] + t2[(uint16_t)(key >> 32)] +
                t3[key >> 48];
    }
  }
  return NULL;
}

/* rows [0,n) split so that every thread gets about the same number of pairs */
static void orc_triangle_split(int32_t n, int nthreads, int32_t *bounds)
{
  double total = (double)n * (n + 1) / 2.0;
  bounds[0] = 0;
  for (int t = 1; t < nthreads; ++t) {
    double target = total * t / nthreads;
    int32_t r = (int32_t)((sqrt(8.0 * target + 1.0) - 1.0) / 2.0);
    if (r < bounds[t - 1]) r = bounds[t - 1];
    if (r > n) r = n;
    bounds[t] = r;
  }
  bounds[nthreads] = n;
}

void orc_gram_lookup(const uint8_t *records, int64_t rlen, const int32_t *cols, int32_t ncols,
                     const uint8_t *killed, const double *tab, const int32_t *xindex, int32_t n,
                     int nthreads, double *XTX)
{
  if (nthreads < 1) nthreads = 1;
  if (nthreads > ORC_MAXTHREADS) nthreads = ORC_MAXTHREADS;
  if (nthreads > n / 2 && n >= 2) nthreads = n / 2 > 0 ? n / 2 : 1;
  uint64_t *geno = (uint64_t *)calloc((size_t)n, sizeof(uint64_t));
  uint64_t *mask = (uint64_t *)calloc((size_t)n, sizeof(uint64_t));
  double *tabs = (double *)calloc(4 * 32768, sizeof(double));
  double *tri = (double *)calloc((size_t)n * (n + 1) / 2, sizeof(double));
  double tb[20][3];
  int32_t bounds[ORC_MAXTHREADS + 1];
  pthread_t th[ORC_MAXTHREADS];
  orc_lookup_job jobs[ORC_MAXTHREADS];
  orc_triangle_split(n, nthreads, bounds);
  int x = 0;
  memset(tb, 0, sizeof tb);
  for (int32_t c = 0; c <= ncols; ++c) {
    int flush = (c == ncols) ? (x > 0) : 0;
    if (c < ncols) {
      if (killed[c]) continue;
      const uint8_t *rec = records + (int64_t)cols[c] * rlen;
      uint32_t sh = 3 * x + x / 5;
      for (int32_t r = 0; r < n; ++r) {
        int g = orc_geno(rec, xindex[r]);
        if (g < 0)
          mask[r] |= (uint64_t)7 << sh;
        else if (g == 1)
          geno[r] |= (uint64_t)2 << sh;
        else if (g == 2)
          geno[r] |= (uint64_t)3 << sh;
      }
      tb[x][0] = tab[4 * c];
      tb[x][1] = tab[4 * c + 1];
      tb[x][2] = tab[4 * c + 2];
      if (++x == 20) flush = 1;
    }
    if (!flush) continue;
    /* tables: field value -> product, summed over the 5 SNPs of each 16-bit slice */
    for (int q = 0; q < 4; ++q) {
      double inc[5][8];
      for (int u = 0; u < 5; ++u) {
        const double *t = tb[5 * q + u];
        inc[u][0] = t[0] * t[0];
        inc[u][1] = 0.0;
        inc[u][2] = t[0] * t[1];
        inc[u][3] = t[0] * t[2];
        inc[u][4] = t[1] * t[1];
        inc[u][5] = t[1] * t[2];
        inc[u][6] = t[2] * t[2];
        inc[u][7] = 0.0;
      }
      double *dst = tabs + 32768 * q;
      for (int a = 0; a < 8; ++a)
        for (int b = 0; b < 8; ++b)
          for (int cc = 0; cc < 8; ++cc)
            for (int d = 0; d < 8; ++d)
              for (int e = 0; e < 8; ++e)
                dst[(a << 12) | (b << 9) | (cc << 6) | (d << 3) | e] =
                    inc[4][a] + inc[3][b] + inc[2][cc] + inc[1][d] + inc[0][e];
    }
    for (int t = 0; t < nthreads; ++t) {
      jobs[t].geno = geno;
      jobs[t].mask = mask;
      jobs[t].tabs = tabs;
      jobs[t].xtx = tri;
      jobs[t].row_lo = bounds[t];
      jobs[t].row_hi = bounds[t + 1];
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, orc_lookup_worker, &jobs[t]);
    orc_lookup_worker(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    memset(geno, 0, sizeof(uint64_t) * (size_t)n);
    memset(mask, 0, sizeof(uint64_t) * (size_t)n);
    memset(tb, 0, sizeof tb);
    x = 0;
  }
  /* symit2 (smartpca.c:480-508): packed lower triangle -> full symmetric */
  for (int32_t i = 0; i < n; ++i)
    for (int32_t j = 0; j <= i; ++j) {
      double v = tri[((int64_t)i * (i + 1)) / 2 + j];
      XTX[(int64_t)i * n + j] = v;
      XTX[(int64_t)j * n + i] = v;
    }
  free(geno);
  free(mask);
  free(tabs);
  free(tri);
}

/* ---- outliers ------------------------------------------------------------------------- */

/* ridoutlier (src/eigensrc/smartsubs.c:18-91), mode 0 and 1; returns the flagged count. */
int orc_ridoutlier(const double *evecs, int32_t n, int32_t neigs, double thresh, int mode,
                   int32_t *badlist, int32_t *vecno, double *score)
{
  if (mode > 1 || n < 3) return 0;
  double *ww = (double *)malloc(sizeof(double) * (size_t)n);
  double *w2 = (double *)malloc(sizeof(double) * (size_t)n);
  int *vbad = (int *)calloc((size_t)n, sizeof(int));
  for (int32_t j = 0; j < n; ++j) vecno[j] = -1, score[j] = 0.0;
  for (int32_t i = 0; i < neigs; ++i) {
    memcpy(ww, evecs + (int64_t)i * n, sizeof(double) * (size_t)n);
    if (mode == 0) {
      double y1 = 0.0, y2 = 0.0;
      for (int32_t j = 0; j < n; ++j) y1 += ww[j];
      y1 /= (double)n;
      for (int32_t j = 0; j < n; ++j) ww[j] = ww[j] + (-y1);
      for (int32_t j = 0; j < n; ++j) y2 += ww[j] * ww[j];
      y2 = sqrt(y2 / (double)n);
      double inv = 1.0 / y2;
      for (int32_t j = 0; j < n; ++j) {
        ww[j] = ww[j] * inv;
        if (fabs(ww[j]) > thresh) {
          vbad[j] = 1;
          if (vecno[j] < 0) vecno[j] = i, score[j] = ww[j];
        }
      }
    } else {
      for (int32_t j = 0; j < n; ++j) {
        double yy = ww[j], y1 = 0.0, y2 = 0.0;
        ww[j] = 0;
        for (int32_t t = 0; t < n; ++t) y1 += ww[t];
        y1 /= (double)(n - 1);
        for (int32_t t = 0; t < n; ++t) w2[t] = ww[t] + (-y1);
        w2[j] = 0;
        for (int32_t t = 0; t < n; ++t) y2 += w2[t] * w2[t];
        y2 = sqrt(y2 / (double)n);
        double zz = (yy - y1) / y2;
        if (fabs(zz) > thresh) {
          vbad[j] = 1;
          if (vecno[j] < 0) vecno[j] = i, score[j] = zz;
        }
        ww[j] = yy;
      }
    }
  }
  int nbad = 0;
  for (int32_t j = 0; j < n; ++j)
    if (vbad[j]) badlist[nbad++] = j;
  free(ww);
  free(w2);
  free(vbad);
  return nbad;
}

/* ---- SNP weights, sample scores, lsqproject ---------------------------------------------- */

/*
 * smartpca.c:1485-1525: ffvecs[j*ncols+c] = sum_k 10 evec_j[k] * v_c[k] (getcolxf column,
 * killed -> 0); fxvecs[j*n+i] = xrow_i . ffvecs_j with fixxrow values g*fancy - xmean;
 * fxscal_j = 1/sqrt(sum_i fxvecs^2).
 */
void orc_weights(const uint8_t *records, int64_t rlen, const int32_t *cols, int32_t ncols,
                 const uint8_t *killed, const double *tab, const double *xmean,
                 const double *xfancy, const int32_t *xindex, int32_t n, const double *evecs,
                 int32_t K, double *ffvecs, double *fxvecs, double *fxscal)
{
  memset(ffvecs, 0, sizeof(double) * (size_t)K * ncols);
  memset(fxvecs, 0, sizeof(double) * (size_t)K * n);
  for (int32_t c = 0; c < ncols; ++c) {
    if (killed[c]) continue;
    const uint8_t *rec = records + (int64_t)cols[c] * rlen;
    for (int32_t k = 0; k < n; ++k) {
      int g = orc_geno(rec, xindex[k]);
      double v = tab[4 * c + (g < 0 ? 3 : g)];
      for (int32_t j = 0; j < K; ++j) ffvecs[(int64_t)j * ncols + c] += (evecs[(int64_t)j * n + k] * 10.0) * v;
    }
  }
  for (int32_t i = 0; i < n; ++i) {
    for (int32_t c = 0; c < ncols; ++c) {
      if (killed[c]) continue;
      int g = orc_geno(records + (int64_t)cols[c] * rlen, xindex[i]);
      if (g < 0) continue;
      double x = (double)g * xfancy[c];
      x = (x < -0.001) ? 0.0 : x - xmean[c];
      for (int32_t j = 0; j < K; ++j) fxvecs[(int64_t)j * n + i] += x * ffvecs[(int64_t)j * ncols + c];
    }
  }
  for (int32_t j = 0; j < K; ++j) {
    double s = 0.0;
    for (int32_t i = 0; i < n; ++i) s += fxvecs[(int64_t)j * n + i] * fxvecs[(int64_t)j * n + i];
    fxscal[j] = 1.0 / sqrt(s);
  }
}

/* choldc / cholsl (src/nicksrc/linsubs.c:331-380); returns -1 when not positive definite */
static int orc_cholsolve(double *a, int K, const double *b, double *x)
{
  double p[64];
  for (int i = 0; i < K; ++i)
    for (int j = i; j < K; ++j) {
      double sum = a[i * K + j];
      for (int k = i - 1; k >= 0; --k) sum -= a[i * K + k] * a[j * K + k];
      if (i == j) {
        if (sum <= 0.0) return -1;
        p[i] = sqrt(sum);
      } else {
        a[j * K + i] = sum / p[i];
      }
    }
  for (int i = 0; i < K; ++i) {
    double sum = b[i];
    for (int k = i - 1; k >= 0; --k) sum -= a[i * K + k] * x[k];
    x[i] = sum / p[i];
  }
  for (int i = K - 1; i >= 0; --i) {
    double sum = x[i];
    for (int k = i + 1; k < K; ++k) sum -= a[k * K + i] * x[k];
    x[i] = sum / p[i];
  }
  return 0;
}

/*
 * lsqproj (smartpca.c:4606-4757) + regressit (src/regsubs.c:8-72) for the listed samples:
 * over kept columns where the sample has a genotype, E_kj = fxscal_j ffvecs_jk,
 * rhs = g*fancy - xmean; co = E^T E, rr = E^T rhs; Cholesky solve.  status 1 when
 * nobs <= K (dropped), 2 when not positive definite (acoeffs untouched).
 * bcoeffs_j = fxscal_j (xrow . ffvecs_j).
 */
void orc_lsqproj(const uint8_t *records, int64_t rlen, const int32_t *cols, int32_t ncols,
                 const uint8_t *killed, const double *xmean, const double *xfancy,
                 const double *ffvecs, const double *fxscal, int32_t K, const int32_t *samples,
                 int32_t nproj, double *acoeffs, double *bcoeffs, int32_t *nobs,
                 int32_t *status)
{
  double co[64 * 64], rr[64], ans[64], e[64];
  for (int32_t q = 0; q < nproj; ++q) {
    memset(co, 0, sizeof(double) * (size_t)K * K);
    memset(rr, 0, sizeof(double) * (size_t)K);
    double bsum[64];
    memset(bsum, 0, sizeof bsum);
    int32_t kk = 0;
    for (int32_t c = 0; c < ncols; ++c) {
      if (killed[c]) continue;
      int g = orc_geno(records + (int64_t)cols[c] * rlen, samples[q]);
      if (g < 0) continue;
      double x = (double)g * xfancy[c];
      x = (x < -0.001) ? 0.0 : x - xmean[c];
      for (int j = 0; j < K; ++j) {
        e[j] = fxscal[j] * ffvecs[(int64_t)j * ncols + c];
        bsum[j] += x * ffvecs[(int64_t)j * ncols + c];
      }
      for (int j = 0; j < K; ++j) {
        rr[j] += e[j] * x;
        for (int k = j; k < K; ++k) co[j * K + k] = co[k * K + j] += e[j] * e[k];
      }
      ++kk;
    }
    nobs[q] = kk;
    for (int j = 0; j < K; ++j) bcoeffs[(int64_t)j * nproj + q] = fxscal[j] * bsum[j];
    if (kk <= K) {
      status[q] = 1;
      continue;
    }
    if (orc_cholsolve(co, K, rr, ans) < 0) {
      status[q] = 2;
      continue;
    }
    for (int j = 0; j < K; ++j) acoeffs[(int64_t)j * nproj + q] = ans[j];
    status[q] = 0;
  }
}

/* ---- usepopsformissing ------------------------------------------------------------------ */

/*
 * getcolxz with usepopsformissing (src/eigensrc/smartpca.c:3129-3216) and fvadjust
 * (:2236-2279), per column over the rows in order: a missing genotype of a row whose
 * population (rowpop, the xtypes index; < 0 = none) has observed genotypes in this column
 * becomes that population's mean genotype; the mean and the fancy scale then run over the
 * observed and filled values in row order.  Outputs (per column): n0, n1 (observed counts),
 * nmiss (still missing after the fill), killed (the rule of :1131-1144 on those counts),
 * gtab [4*c] (k - mean)*fancy, gfill [c*npop + k] (fill_k - mean)*fancy (0 where population
 * k has no observed genotype), xmean = mean*fancy, xfancy = fancy.  A column with no
 * observed genotype: n0 = n1 = -1, nmiss = nrows, killed, xmean = xfancy = 0.
 */
void orc_popfill_columns(const uint8_t *records, int64_t rlen, const int32_t *cols,
                         int32_t ncols, const int32_t *xindex, int32_t nrows,
                         const int32_t *rowpop, int32_t npop, int fancynorm, int altnormstyle,
                         int minallelecnt, int maxmissing, int32_t *n0, int32_t *n1,
                         int32_t *nmiss, uint8_t *killed, double *gtab, double *gfill,
                         double *xmean, double *xfancy)
{
  double *psum = (double *)malloc(sizeof(double) * (size_t)(npop + 1));
  double *pnum = (double *)malloc(sizeof(double) * (size_t)(npop + 1));
  double *x = (double *)malloc(sizeof(double) * (size_t)(nrows + 1));
  for (int32_t c = 0; c < ncols; ++c) {
    const uint8_t *rec = records + (int64_t)cols[c] * rlen;
    double *tab = gtab + 4 * (int64_t)c, *fill = gfill + (int64_t)c * npop;
    memset(psum, 0, sizeof(double) * (size_t)npop);
    memset(pnum, 0, sizeof(double) * (size_t)npop);
    int c0 = 0, c1 = 0, miss = 0;
    for (int32_t j = 0; j < nrows; ++j) {
      const int g = orc_geno(rec, xindex[j]);
      x[j] = (double)g;
      if (g < 0) {
        ++miss;
        continue;
      }
      c0 += g;
      c1 += 2 - g;
      const int k = rowpop[j];
      if (k >= 0) {
        psum[k] += (double)g;
        pnum[k] += 1.0;
      }
    }
    if (miss > 0) {
      miss = 0;
      for (int32_t j = 0; j < nrows; ++j) {
        if (x[j] >= 0.0) continue;
        const int k = rowpop[j];
        if (k >= 0 && pnum[k] > 0.5) x[j] = psum[k] / pnum[k];
        else ++miss;
      }
    }
    double ysum = 0.0, ynum = 0.0;
    for (int32_t j = 0; j < nrows; ++j)
      if (x[j] >= 0.0) {
        ysum += x[j];
        ynum += 1.0;
      }
    for (int k = 0; k < npop; ++k) fill[k] = 0.0;
    tab[0] = tab[1] = tab[2] = tab[3] = 0.0;
    if (ynum == 0.0) {
      n0[c] = n1[c] = -1;
      nmiss[c] = nrows;
      killed[c] = 1;
      xmean[c] = xfancy[c] = 0.0;
      continue;
    }
    const double ymean = ysum / ynum;
    double yfancy = 1.0;
    if (fancynorm) {
      double p = 0.5 * ymean;
      if (altnormstyle == 0) p = (ysum + 1.0) / (2.0 * ynum + 2.0);
      const double y = p * (1.0 - p);
      if (y > 0.0) yfancy = 1.0 / sqrt(y);
    }
    n0[c] = c0;
    n1[c] = c1;
    nmiss[c] = miss;
    xmean[c] = ymean * yfancy;
    xfancy[c] = yfancy;
    const int t = c0 < c1 ? c0 : c1;
    killed[c] = (t < minallelecnt) || (miss > maxmissing) || (t == 0);
    if (killed[c]) continue;
    for (int g = 0; g < 3; ++g) tab[g] = ((double)g - ymean) * yfancy;
    for (int k = 0; k < npop; ++k)
      if (pnum[k] > 0.5) fill[k] = (psum[k] / pnum[k] - ymean) * yfancy;
  }
  free(psum);
  free(pnum);
  free(x);
}

/* XTX with the usepopsformissing values: the table for observed genotypes, the row's
 * population fill (0 without one) for missing ones (smartpca.c:1116-1189 through getcolxz
 * and domult_increment_normal :3498-3561); plain loops, lower triangle then mirrored. */
void orc_gram_fill(const uint8_t *records, int64_t rlen, const int32_t *cols, int32_t ncols,
                   const uint8_t *killed, const double *gtab, const double *gfill, int32_t npop,
                   const int32_t *rowpop, const int32_t *xindex, int32_t n, double *XTX)
{
  double *v = (double *)malloc(sizeof(double) * (size_t)n);
  memset(XTX, 0, sizeof(double) * (size_t)n * n);
  for (int32_t c = 0; c < ncols; ++c) {
    if (killed[c]) continue;
    const uint8_t *rec = records + (int64_t)cols[c] * rlen;
    for (int32_t i = 0; i < n; ++i) {
      const int g = orc_geno(rec, xindex[i]);
      v[i] = g >= 0 ? gtab[4 * (int64_t)c + g]
                    : (rowpop[i] >= 0 ? gfill[(int64_t)c * npop + rowpop[i]] : 0.0);
    }
    for (int32_t i = 0; i < n; ++i) {
      const double vi = v[i];
      if (vi == 0.0) continue;
      double *row = XTX + (int64_t)i * n;
      for (int32_t j = 0; j <= i; ++j) row[j] += vi * v[j];
    }
  }
  for (int32_t i = 0; i < n; ++i)
    for (int32_t j = i + 1; j < n; ++j) XTX[(int64_t)i * n + j] = XTX[(int64_t)j * n + i];
  free(v);
}

/*
 * lsqproj with usepopsformissing (src/eigensrc/smartpca.c:4606-4757).  sampop[q] is the
 * population index the reference reads for sample q (xtypes[idnum]; < 0 = none).  A sample
 * with at most K observed genotypes over the kept columns is "ignored (insufficient data"
 * (status 1, the first-call coverage check :4631-4647) and adds nothing to the population
 * sums; the others with sampop >= 0 sum their observed genotypes per population and column
 * (xnum, xden :4658-4677).  Each sample's missing genotypes are then filled with its
 * population's mean where xden > 0.1 and count as observed in the regression (:4679-4716)
 * and in bcoeffs (:4719-4746); fixxrow values (x fancy - xmean).
 */
void orc_lsqproj_fill(const uint8_t *records, int64_t rlen, const int32_t *cols, int32_t ncols,
                      const uint8_t *killed, const double *xmean, const double *xfancy,
                      const double *ffvecs, const double *fxscal, int32_t K,
                      const int32_t *samples, const int32_t *sampop, int32_t nproj,
                      int32_t npop, double *acoeffs, double *bcoeffs, int32_t *nobs,
                      int32_t *status)
{
  double co[64 * 64], rr[64], ans[64], e[64], bsum[64];
  double *xnum = (double *)calloc((size_t)npop * ncols + 1, sizeof(double));
  double *xden = (double *)calloc((size_t)npop * ncols + 1, sizeof(double));
  int32_t *raw = (int32_t *)calloc((size_t)nproj + 1, sizeof(int32_t));
  for (int32_t q = 0; q < nproj; ++q)
    for (int32_t c = 0; c < ncols; ++c)
      if (!killed[c] && orc_geno(records + (int64_t)cols[c] * rlen, samples[q]) >= 0) ++raw[q];
  for (int32_t q = 0; q < nproj; ++q) {
    const int t = sampop[q];
    if (raw[q] <= K || t < 0) continue;
    for (int32_t c = 0; c < ncols; ++c) {
      const int g = orc_geno(records + (int64_t)cols[c] * rlen, samples[q]);
      if (g < 0) continue;
      xnum[(int64_t)t * ncols + c] += (double)g;
      xden[(int64_t)t * ncols + c] += 1.0;
    }
  }
  for (int32_t q = 0; q < nproj; ++q) {
    const int t = sampop[q];
    memset(co, 0, sizeof(double) * (size_t)K * K);
    memset(rr, 0, sizeof(double) * (size_t)K);
    memset(bsum, 0, sizeof bsum);
    if (raw[q] <= K) {
      nobs[q] = raw[q];
      status[q] = 1;
      for (int j = 0; j < K; ++j) bcoeffs[(int64_t)j * nproj + q] = 0.0;
      continue;
    }
    int32_t kk = 0;
    for (int32_t c = 0; c < ncols; ++c) {
      if (killed[c]) continue;
      const int g = orc_geno(records + (int64_t)cols[c] * rlen, samples[q]);
      double xr = (double)g;
      if (g < 0) {
        const int64_t u = (int64_t)t * ncols + c;
        if (t < 0 || !(xden[u] > 0.1)) continue;
        xr = xnum[u] / xden[u];
      }
      double x = xr * xfancy[c];
      x = (x < -0.001) ? 0.0 : x - xmean[c];
      for (int j = 0; j < K; ++j) {
        e[j] = fxscal[j] * ffvecs[(int64_t)j * ncols + c];
        bsum[j] += x * ffvecs[(int64_t)j * ncols + c];
      }
      for (int j = 0; j < K; ++j) {
        rr[j] += e[j] * x;
        for (int k = j; k < K; ++k) co[j * K + k] = co[k * K + j] += e[j] * e[k];
      }
      ++kk;
    }
    nobs[q] = kk;
    for (int j = 0; j < K; ++j) bcoeffs[(int64_t)j * nproj + q] = fxscal[j] * bsum[j];
    if (orc_cholsolve(co, K, rr, ans) < 0) {
      status[q] = 2;
      continue;
    }
    for (int j = 0; j < K; ++j) acoeffs[(int64_t)j * nproj + q] = ans[j];
    status[q] = 0;
  }
  free(xnum);
  free(xden);
  free(raw);
}
