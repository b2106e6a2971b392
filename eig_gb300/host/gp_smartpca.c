/*
 * The smartpca flow over the gpupca C ABI, host side in C.  It restates the control flow
 * of main() in src/eigensrc/smartpca.c for the hot path and calls the device entry points
 * where the reference calls its compute functions:
 *
 *   SNP pre-filters (chrom X/0/big :801-824, nodata :826-850), samples without data
 *   (:869-881), loadindx/loadsnpx (:936-937), the outlier loop (:1077-1265: gp_xtx,
 *   gp_eigvecs, gp_ridoutlier), SNP weights (:1485-1525: gp_snp_weights), lsqproj
 *   (:1553: gp_lsqproj) with seteigscale (:4758-4782) and the rescale (:1556-1564), and
 *   fastmode (:950-980: gp_fastpca, printevecs normalisation :3845-3871);
 *   usepopsformissing: the xtypes array (:928-943, :1095-1099, :1505-1508) handed to
 *   gp_set_row_pops per pass and, indexed by the sample's .ind position as lsqproj reads it
 *   (:4658-4690), to gp_lsqproj_pops.
 *
 * Parfile parsing and the .evec/.eval text live in the CLI (gpusmartpca_main.c); this file
 * works on in-memory arrays so the same flow serves the CLI and the ctypes callers.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/gpupca.h"
#include "../../include/gpupca_run.h"

static double now_s(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

void gp_smartpca_defaults(gp_smartpca_opts *o)
{
  memset(o, 0, sizeof *o);
  o->numeigs = 10;       /* smartpca.c:164 */
  o->numoutliter = 5;    /* :211 */
  o->numoutleigs = 10;
  o->outlthresh = 6.0;   /* :212 */
  o->outliermode = 0;
  o->fancynorm = 1;      /* include/globals.h:5 */
  o->altnormstyle = 1;   /* :186 */
  o->minallelecnt = 1;
  o->maxmissing = 9999999;
  o->lsqproject = 1;     /* :208 regmode */
  o->noxdata = 1;
  o->numchrom = 22;
  o->precision = GP_PREC_FP64;
  o->fastmode = 0;
  o->fastdim = -1;
  o->fastiter = -1;
  o->seed = 0;
  o->missingmode = 0;
  o->usepopsformissing = 0;
}

static int geno_at(const gp_panel *p, int64_t s, int32_t k)
{
  const uint8_t *rec = p->records + s * p->record_bytes;
  int g;
  if (p->code == GP_CODE_BED) {
    int x = (rec[k >> 2] >> ((k & 3) * 2)) & 3;
    g = (x == 0) ? 2 : (x == 1) ? -1 : (x == 2) ? 1 : 0;
  } else {
    g = (rec[k >> 2] >> ((3 - (k & 3)) * 2)) & 3;
    if (g == 3) g = -1;
  }
  return g;
}

#define FAIL(code_)   \
  do {                \
    rc = (code_);     \
    goto done;        \
  } while (0)

int gp_smartpca_run(gp_ctx *ctx, const gp_smartpca_opts *o, const gp_panel *p,
                    gp_run_result *r)
{
  int rc = GP_OK;
  const int64_t M = p->nsnp;
  const int32_t N = p->nind;
  double t0 = now_s(), t;
  uint8_t *snp_ign = NULL, *ind_ign = NULL, *aff = NULL, *use = NULL, *kill = NULL;
  int32_t *valid_s = NULL, *valid_i = NULL, *xindex = NULL, *cols = NULL, *badlist = NULL;
  int32_t *vecno = NULL, *nobs = NULL, *status = NULL, *projidx = NULL, *xtypes = NULL;
  int32_t *pc0 = NULL, *pc1 = NULL, *pcm = NULL; /* per-column counts for pass_stats */
  int32_t *sampop = NULL, npop = 0;
  double *evals = NULL, *evecs = NULL, *score = NULL, *fxscal = NULL, *acoef = NULL,
         *bcoef = NULL;
  memset(r->t_phase, 0, sizeof r->t_phase);
  r->noutliers = 0;
  r->npasses = 0;
  r->gram_flops = 0.0;
  r->gram_ms = 0.0;
  r->nused = 0;
  if (!ctx || !o || !p || !r || M < 1 || N < 1) return GP_ERR_ARG;

  snp_ign = (uint8_t *)calloc((size_t)M, 1);
  ind_ign = (uint8_t *)calloc((size_t)N, 1);
  aff = (uint8_t *)calloc((size_t)N, 1);
  use = (uint8_t *)calloc((size_t)(M > N ? M : N), 1);
  kill = (uint8_t *)calloc((size_t)M, 1);
  valid_s = (int32_t *)calloc((size_t)M, sizeof(int32_t));
  valid_i = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  xindex = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  cols = (int32_t *)calloc((size_t)M, sizeof(int32_t));
  badlist = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  vecno = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  score = (double *)calloc((size_t)N, sizeof(double));
  if (!snp_ign || !ind_ign || !aff || !use || !kill || !valid_s || !valid_i || !xindex || !cols ||
      !badlist || !vecno || !score)
    FAIL(GP_ERR_NOMEM);
  if (o->usepopsformissing) {
    if (!p->ind_pop)
      FAIL(gp_fail_msg(ctx, GP_ERR_ARG, "usepopsformissing needs the samples' populations"));
    if (o->precision != GP_PREC_FP64)
      FAIL(gp_fail_msg(ctx, GP_ERR_ARG, "usepopsformissing runs in FP64 precision only"));
    if (o->fastmode)
      FAIL(gp_fail_msg(ctx, GP_ERR_ARG, "usepopsformissing with fastmode is not supported"));
    /* xtypes[i]: population of row i, written for the rows of every pass and never cleared
     * (-2 before the first), as the reference keeps it */
    xtypes = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    sampop = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    if (!xtypes || !sampop) FAIL(GP_ERR_NOMEM);
    for (int32_t k = 0; k < N; ++k) {
      xtypes[k] = -2;
      if (p->ind_pop[k] >= npop) npop = p->ind_pop[k] + 1;
    }
    if (npop < 1) npop = 1;
  }

  /* ---- upload (inpack / getbedgenos) and the male-X-het rule -------------------------- */
  if (p->records) {
    rc = gp_load_genotypes(ctx, p->records, p->record_bytes, M, N, p->code);
    if (rc) goto done;
  } else {
    /* resident panel: the records were uploaded by an earlier gp_load_genotypes */
    int64_t rs = 0;
    int32_t rn = 0;
    gp_genotype_shape(ctx, &rs, &rn);
    if (rs != M || rn != N)
      FAIL(gp_fail_msg(ctx, GP_ERR_STATE, "resident panel is %lld x %d, run asks %lld x %d",
                       (long long)rs, rn, (long long)M, N));
  }
  if (p->records && !o->noxdata && p->ind_male && p->snp_chrom) {
    /* checkxval: male het on chrom X -> missing (src/mcio.c:1606-1619, :2856-2863) */
    int64_t cap = 1024, np = 0;
    int64_t *pairs = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)cap);
    if (!pairs) FAIL(GP_ERR_NOMEM);
    for (int64_t s = 0; s < M; ++s) {
      if (p->snp_chrom[s] != o->numchrom + 1) continue;
      for (int32_t k = 0; k < N; ++k) {
        if (!p->ind_male[k] || geno_at(p, s, k) != 1) continue;
        if (np == cap) {
          cap *= 2;
          int64_t *nb = (int64_t *)realloc(pairs, sizeof(int64_t) * 2 * (size_t)cap);
          if (!nb) {
            free(pairs);
            FAIL(GP_ERR_NOMEM);
          }
          pairs = nb;
        }
        pairs[2 * np] = s;
        pairs[2 * np + 1] = k;
        ++np;
      }
    }
    rc = gp_set_missing(ctx, pairs, np);
    free(pairs);
    if (rc) goto done;
  }
  t = now_s();
  r->t_phase[GP_PH_LOAD] = t - t0;

  /* ---- pre-filters -------------------------------------------------------------------- */
  for (int32_t k = 0; k < N; ++k) {
    ind_ign[k] = p->ind_ignore ? p->ind_ignore[k] : 0;
    aff[k] = ind_ign[k] ? 0 : (p->ind_affstatus ? p->ind_affstatus[k] : 1);
  }
  for (int64_t s = 0; s < M; ++s) {
    int ch = p->snp_chrom ? p->snp_chrom[s] : 1;
    snp_ign[s] = p->snp_ignore ? p->snp_ignore[s] : 0;
    if (snp_ign[s]) continue;
    if (o->noxdata && ch == o->numchrom + 1) snp_ign[s] = 1;      /* chrom-X */
    else if (ch == 0) snp_ign[s] = 1;                               /* chrom-0 */
    else if (ch > o->numchrom + 1) snp_ign[s] = 1;                  /* chrom-big */
  }
  /* nodata: numvalidgtx over non-ignored samples with affstatus YES, <= 1 -> ignore */
  for (int32_t k = 0; k < N; ++k) use[k] = (uint8_t)(!ind_ign[k] && aff[k]);
  rc = gp_valid_counts(ctx, use, NULL, valid_s, NULL);
  if (rc) goto done;
  r->nodata = 0;
  for (int64_t s = 0; s < M; ++s)
    if (!snp_ign[s] && valid_s[s] <= 1) {
      snp_ign[s] = 1;
      ++r->nodata;
    }
  /* samples with no valid genotype over the remaining SNPs -> ignore (numvalidgtallind) */
  for (int64_t s = 0; s < M; ++s) use[s] = (uint8_t)!snp_ign[s];
  rc = gp_valid_counts(ctx, NULL, use, NULL, valid_i);
  if (rc) goto done;
  for (int32_t k = 0; k < N; ++k)
    if (valid_i[k] == 0) ind_ign[k] = 1;

  int32_t nrows = 0, ncols = 0;
  for (int32_t k = 0; k < N; ++k)
    if (!ind_ign[k] && aff[k]) xindex[nrows++] = k;
  /* missingmode (smartpca.c:901-904): setmiss after the pre-filters, then no fancynorm */
  gp_smartpca_opts om = *o;
  if (o->missingmode) {
    rc = gp_set_missingmode(ctx);
    if (rc) goto done;
    om.fancynorm = 0;
  }
  o = &om;
  /* loadsnpx: non-ignored SNPs with a valid genotype among non-ignored samples */
  for (int32_t k = 0; k < N; ++k) use[k] = (uint8_t)!ind_ign[k];
  rc = gp_valid_counts(ctx, use, NULL, valid_s, NULL);
  if (rc) goto done;
  for (int64_t s = 0; s < M; ++s)
    if (!snp_ign[s] && valid_s[s] > 0) cols[ncols++] = (int32_t)s;
  if (nrows < 2 || ncols < 1) FAIL(gp_fail_msg(ctx, GP_ERR_NODATA, "no data (rows %d, snps %d)", nrows, ncols));
  r->nrows0 = nrows;
  r->ncols0 = ncols;
  r->t_phase[GP_PH_FILTER] = now_s() - t;

  int32_t K = o->numeigs;

  /* ---- fastmode ----------------------------------------------------------------------- */
  if (o->fastmode && K > 0) {
    int32_t L = o->fastdim < 0 ? 2 * K : o->fastdim;
    int32_t I = o->fastiter < 0 ? K : o->fastiter;
    t = now_s();
    rc = gp_set_samples(ctx, xindex, nrows);
    if (!rc) rc = gp_set_snps(ctx, cols, ncols);
    if (rc) goto done;
    evals = (double *)calloc((size_t)K, sizeof(double));
    evecs = (double *)calloc((size_t)K * nrows, sizeof(double));
    if (!evals || !evecs) FAIL(GP_ERR_NOMEM);
    gp_xtx_opts fo = {o->fancynorm, o->altnormstyle, 0, 0x7fffffff, o->precision};
    rc = gp_fastpca(ctx, K, L, I, (uint64_t)o->seed, NULL, &fo, evals, evecs);
    if (rc) goto done;
    r->t_phase[GP_PH_GRAM] = now_s() - t;
    r->nrows = nrows;
    r->ncols = ncols;
    r->numeigs = K;
    r->npasses = 1;
    memcpy(r->xindex, xindex, sizeof(int32_t) * (size_t)nrows);
    memcpy(r->evals, evals, sizeof(double) * (size_t)K);
    memset(r->ind_out, 0, (size_t)N);
    for (int32_t j = 0; j < K; ++j) {
      /* printevecs: fvecs = 10 evec normalised to unit length (:3845-3871) */
      double s = 0.0;
      for (int32_t i = 0; i < nrows; ++i) {
        double v = evecs[(size_t)j * nrows + i] * 10.0;
        s += v * v;
      }
      double inv = 1.0 / sqrt(s);
      for (int32_t i = 0; i < nrows; ++i) {
        double v = (evecs[(size_t)j * nrows + i] * 10.0) * inv;
        r->evecs[(size_t)j * nrows + i] = evecs[(size_t)j * nrows + i];
        r->coords[(size_t)j * N + xindex[i]] = v;
      }
    }
    for (int32_t i = 0; i < nrows; ++i) r->ind_out[xindex[i]] = 1;
    for (int64_t s = 0; s < M; ++s) r->snp_state[s] = snp_ign[s] ? 1 : 0;
    r->t_phase[GP_PH_TOTAL] = now_s() - t0;
    goto done;
  }

  /* ---- outlier loop ------------------------------------------------------------------- */
  evals = (double *)calloc((size_t)N, sizeof(double));
  int32_t nvec_keep = K > o->numoutleigs ? K : o->numoutleigs;
  if (nvec_keep < 1) nvec_keep = 1;
  evecs = (double *)calloc((size_t)nvec_keep * N, sizeof(double));
  if (!evals || !evecs) FAIL(GP_ERR_NOMEM);
  int32_t numoutiter = o->numoutliter >= 1 ? o->numoutliter + 1 : 1;
  int mode = o->numoutliter >= 1 ? o->outliermode : 2;
  int32_t numoutleigs = o->numoutleigs;
  gp_xtx_opts xo;
  xo.fancynorm = o->fancynorm;
  xo.altnormstyle = o->altnormstyle;
  xo.minallelecnt = o->minallelecnt;
  xo.maxmissing = o->maxmissing;
  xo.precision = o->precision;
  if (r->pass_stats) {
    pc0 = (int32_t *)malloc(sizeof(int32_t) * (size_t)M);
    pc1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)M);
    pcm = (int32_t *)malloc(sizeof(int32_t) * (size_t)M);
    if (!pc0 || !pc1 || !pcm) FAIL(GP_ERR_NOMEM);
  }
  for (int32_t it = 1; it <= numoutiter; ++it) {
    if (it > 1) {
      for (int32_t k = 0; k < N; ++k) use[k] = (uint8_t)!ind_ign[k];
      rc = gp_valid_counts(ctx, use, NULL, valid_s, NULL);
      if (rc) goto done;
      ncols = 0;
      for (int64_t s = 0; s < M; ++s)
        if (!snp_ign[s] && valid_s[s] > 0) cols[ncols++] = (int32_t)s;
      if (ncols < 1) FAIL(gp_fail_msg(ctx, GP_ERR_NODATA, "no SNPs left"));
    }
    t = now_s();
    rc = gp_set_samples(ctx, xindex, nrows);
    if (!rc) rc = gp_set_snps(ctx, cols, ncols);
    if (!rc && xtypes) {
      for (int32_t i = 0; i < nrows; ++i) xtypes[i] = p->ind_pop[xindex[i]];
      rc = gp_set_row_pops(ctx, xtypes, npop);
    }
    if (rc) goto done;
    double trace;
    int32_t nused;
    rc = gp_xtx(ctx, &xo, pc0, pc1, pcm, kill, NULL, NULL, r->xtx, &trace, &nused);
    if (rc) goto done;
    r->nused = nused;
    if (r->pass_stats) {
      /* the pass's dropped SNPs and its first 10 (smartpca.c:1134-1143) */
      int32_t *ps = r->pass_stats + (size_t)GP_PASS_STATS * (it - 1);
      int32_t *pk = r->pass_kills ? r->pass_kills + (size_t)30 * (it - 1) : NULL;
      int32_t nk = 0, nl = 0;
      for (int32_t c = 0; c < ncols; ++c) {
        if (!kill[c]) continue;
        if (pk && nl < 10) {
          const int32_t mn = pc0[c] < pc1[c] ? pc0[c] : pc1[c];
          pk[3 * nl] = cols[c];
          pk[3 * nl + 1] = mn > 0 ? mn : 0;
          pk[3 * nl + 2] = pcm[c] > 0 ? pcm[c] : 0;
          ++nl;
        }
        ++nk;
      }
      ps[0] = nk;
      ps[1] = nused;
      ps[2] = -1;
      ps[3] = nl;
    }
    {
      double gms = 0.0, gfl = 0.0;
      gp_last_gram_time(ctx, &gms, NULL, &gfl);
      r->gram_ms += gms;
      r->gram_flops += gfl;
    }
    for (int32_t c = 0; c < ncols; ++c)
      if (kill[c]) {
        snp_ign[cols[c]] = 2; /* minallelecnt: ignored from now on */
      }
    double tg = now_s();
    r->t_phase[GP_PH_GRAM] += tg - t;
    int32_t nv = nvec_keep < nrows ? nvec_keep : nrows;
    rc = gp_eigvecs(ctx, nv, evals, evecs);
    if (rc) goto done;
    double te = now_s();
    r->t_phase[GP_PH_EIG] += te - tg;
    r->npasses = it;
    if (it > o->numoutliter) break;
    if (numoutleigs > nrows - 1) numoutleigs = nrows - 1;
    int32_t nbad = gp_ridoutlier(evecs, nrows, numoutleigs < nv ? numoutleigs : nv, o->outlthresh,
                                 mode, badlist, vecno, score);
    if (nbad < 0) FAIL(nbad);
    r->t_phase[GP_PH_OUTLIER] += now_s() - te;
    if (nbad == 0) break;
    for (int32_t b = 0; b < nbad; ++b) {
      int32_t row = badlist[b];
      int32_t k = xindex[row];
      if (r->outlier_idx && r->noutliers < N) {
        r->outlier_idx[r->noutliers] = k;
        r->outlier_iter[r->noutliers] = it;
        r->outlier_vec[r->noutliers] = vecno[row];
        r->outlier_score[r->noutliers] = score[row];
      }
      r->noutliers++;
      ind_ign[k] = 1;
    }
    nrows = 0;
    for (int32_t k = 0; k < N; ++k)
      if (!ind_ign[k] && aff[k]) xindex[nrows++] = k;
    if (r->pass_stats) r->pass_stats[(size_t)GP_PASS_STATS * (it - 1) + 2] = nrows;
    if (nrows < 2) FAIL(gp_fail_msg(ctx, GP_ERR_NODATA, "outlier removal left %d samples", nrows));
  }

  /* eigenvalues / vectors of the last pass */
  r->nrows = nrows;
  r->ncols = ncols;
  memcpy(r->xindex, xindex, sizeof(int32_t) * (size_t)nrows);
  memcpy(r->evals, evals, sizeof(double) * (size_t)nrows);
  if (K > nrows) K = nrows;
  if (K > ncols) K = ncols;
  r->numeigs = K;
  memcpy(r->evecs, evecs, sizeof(double) * (size_t)K * nrows);
  for (int64_t s = 0; s < M; ++s) r->snp_state[s] = snp_ign[s];
  if (r->snp_lastpass) {
    memset(r->snp_lastpass, 0, (size_t)M);
    for (int32_t c = 0; c < ncols; ++c) r->snp_lastpass[cols[c]] = 1;
  }
  memset(r->ind_out, 0, (size_t)N);
  memset(r->coords, 0, sizeof(double) * (size_t)K * N);
  if (K <= 0) goto done;

  /* ---- SNP weights, lsqproject, eigscale ---------------------------------------------- */
  t = now_s();
  fxscal = (double *)calloc((size_t)K, sizeof(double));
  if (!fxscal) FAIL(GP_ERR_NOMEM);
  if (r->ffvecs) {
    /* the weights over the last pass's columns, scattered to SNP order */
    double *ff = (double *)malloc(sizeof(double) * (size_t)K * ncols);
    if (!ff) FAIL(GP_ERR_NOMEM);
    rc = gp_snp_weights(ctx, K, ff, NULL, fxscal);
    if (!rc) {
      memset(r->ffvecs, 0, sizeof(double) * (size_t)K * M);
      for (int32_t j = 0; j < K; ++j)
        for (int32_t c = 0; c < ncols; ++c)
          r->ffvecs[(size_t)j * M + cols[c]] = ff[(size_t)j * ncols + c];
    }
    free(ff);
  } else {
    rc = gp_snp_weights(ctx, K, NULL, NULL, fxscal);
  }
  if (rc) goto done;
  double tw = now_s();
  r->t_phase[GP_PH_WEIGHTS] = tw - t;
  int32_t nproj = 0;
  projidx = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  if (!projidx) FAIL(GP_ERR_NOMEM);
  for (int32_t k = 0; k < N; ++k)
    if (!ind_ign[k]) projidx[nproj++] = k;
  if (o->lsqproject) {
    acoef = (double *)calloc((size_t)K * nproj, sizeof(double));
    bcoef = (double *)calloc((size_t)K * nproj, sizeof(double));
    nobs = (int32_t *)calloc((size_t)nproj, sizeof(int32_t));
    status = (int32_t *)calloc((size_t)nproj, sizeof(int32_t));
    if (!acoef || !bcoef || !nobs || !status) FAIL(GP_ERR_NOMEM);
    if (xtypes) {
      /* lsqproj reads xtypes at the sample's .ind index (idnum), not at its row */
      for (int32_t q = 0; q < nproj; ++q) sampop[q] = xtypes[projidx[q]];
      rc = gp_lsqproj_pops(ctx, K, projidx, sampop, npop, nproj, acoef, bcoef, nobs, status);
    } else {
      rc = gp_lsqproj(ctx, K, projidx, nproj, acoef, bcoef, nobs, status);
    }
    if (rc) goto done;
    /* the reference keeps the previous regans for a non-PD system (regsubs.c:51-53) */
    double prev[64];
    memset(prev, 0, sizeof prev);
    for (int32_t q = 0; q < nproj; ++q) {
      int32_t k = projidx[q];
      if (status[q] == 1) {
        ind_ign[k] = 1; /* "ignored (insufficient data" */
        continue;
      }
      for (int32_t j = 0; j < K; ++j) {
        if (status[q] == 2) acoef[(size_t)j * nproj + q] = prev[j];
        prev[j] = acoef[(size_t)j * nproj + q];
        r->coords[(size_t)j * N + k] = acoef[(size_t)j * nproj + q];
      }
    }
    /* seteigscale over the PCA rows, then acoeffs *= eigscale (smartpca.c:1556-1564) */
    for (int32_t j = 0; j < K; ++j) {
      double ab = 0.0, aa = 0.0;
      for (int32_t i = 0; i < nrows; ++i) {
        int32_t k = xindex[i];
        /* position of k among the projected samples */
        int32_t lo = 0, hi = nproj - 1, q = -1;
        while (lo <= hi) {
          int32_t mid = (lo + hi) >> 1;
          if (projidx[mid] == k) {
            q = mid;
            break;
          }
          if (projidx[mid] < k) lo = mid + 1;
          else hi = mid - 1;
        }
        double a = 0.0, b = 0.0;
        if (q >= 0 && status[q] != 1) {
          a = r->coords[(size_t)j * N + k];
          b = bcoef[(size_t)j * nproj + q];
        }
        ab += a * b;
        aa += a * a;
      }
      double sc = ab / aa;
      for (int32_t q = 0; q < nproj; ++q) {
        int32_t k = projidx[q];
        r->coords[(size_t)j * N + k] = sc * r->coords[(size_t)j * N + k];
      }
    }
  }
  for (int32_t k = 0; k < N; ++k) r->ind_out[k] = (uint8_t)!ind_ign[k];
  r->t_phase[GP_PH_LSQ] = now_s() - tw;
  r->t_phase[GP_PH_TOTAL] = now_s() - t0;

done:
  free(snp_ign);
  free(ind_ign);
  free(aff);
  free(use);
  free(kill);
  free(valid_s);
  free(valid_i);
  free(xindex);
  free(cols);
  free(badlist);
  free(vecno);
  free(score);
  free(evals);
  free(evecs);
  free(fxscal);
  free(acoef);
  free(bcoef);
  free(nobs);
  free(status);
  free(projidx);
  free(xtypes);
  free(sampop);
  free(pc0);
  free(pc1);
  free(pcm);
  return rc;
}
