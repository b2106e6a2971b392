/*
 * gpupca_run.h — the whole smartpca hot path as one C call (host flow in C over the entry
 * points of gpupca.h).  Replaces the body of main() in src/eigensrc/smartpca.c from the
 * SNP/sample pre-filters (:795-937) through the outlier loop (:1077-1265), SNP weights
 * (:1485-1525), lsqproj + eigscale (:1549-1565) and the fastmode branch (:950-980).
 * Reading the parfile and the genotype files, and writing .evec/.eval, stay in the CLI
 * (gpusmartpca) so that this call works on in-memory arrays.
 */
#ifndef GPUPCA_RUN_H
#define GPUPCA_RUN_H

#include <stdint.h>

#include "gpupca.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t numeigs;      /* numoutevec (default 10) */
  int32_t numoutliter;  /* numoutlieriter (5) */
  int32_t numoutleigs;  /* numoutlierevec (10) */
  double outlthresh;    /* outliersigmathresh (6.0) */
  int32_t outliermode;  /* outliermode (0) */
  int32_t fancynorm;    /* usenorm (YES) */
  int32_t altnormstyle; /* altnormstyle (YES) */
  int32_t minallelecnt; /* minallelecnt (1) */
  int32_t maxmissing;   /* maxmissing (9999999) */
  int32_t lsqproject;   /* lsqproject (YES) */
  int32_t noxdata;      /* noxdata (YES) */
  int32_t numchrom;     /* numchrom (22) */
  int32_t precision;    /* GP_PREC_FP64 (drop-in) or GP_PREC_SPLIT_BF16 */
  int32_t fastmode;     /* fastmode (NO) */
  int32_t fastdim;      /* fastdim (-1: 2*numeigs) */
  int32_t fastiter;     /* fastiter (-1: numeigs) */
  int64_t seed;         /* seed (fastmode Omega) */
  int32_t missingmode;  /* missingmode (NO): PCA of the missingness indicators, no fancynorm */
  int32_t usepopsformissing; /* usepopsformissing (NO): missing -> population mean (FP64
                                precision, not with fastmode; needs gp_panel.ind_pop) */
} gp_smartpca_opts;

typedef struct {
  const uint8_t *records;      /* nsnp records, SNP-major, sorted SNP order; NULL = use the
                                  panel already resident on the handle (gp_load_genotypes) */
  int64_t record_bytes;
  int64_t nsnp;
  int32_t nind;
  int32_t code;                /* GP_CODE_PACKED / GP_CODE_BED */
  const int32_t *snp_chrom;    /* [nsnp] chromosome numbers (X = numchrom+1), NULL = all 1 */
  const uint8_t *snp_ignore;   /* [nsnp] pre-ignored SNPs (badsnpname), may be NULL */
  const uint8_t *ind_ignore;   /* [nind] population "Ignore", may be NULL */
  const uint8_t *ind_affstatus;/* [nind] 1 = in a poplistname population (NULL = all) */
  const uint8_t *ind_male;     /* [nind] 1 = gender M (male-X-het rule), may be NULL */
  const int32_t *ind_pop;      /* [nind] index of the sample's population in the population
                                  list (poplistname order, else first appearance), -1 when
                                  not listed; read only with usepopsformissing */
} gp_panel;

enum {
  GP_PH_LOAD = 0,
  GP_PH_FILTER = 1,
  GP_PH_GRAM = 2,
  GP_PH_EIG = 3,
  GP_PH_OUTLIER = 4,
  GP_PH_WEIGHTS = 5,
  GP_PH_LSQ = 6,
  GP_PH_TOTAL = 7
};

typedef struct {
  /* caller-allocated outputs (sizes in brackets) */
  int32_t *xindex;         /* [nind]  final PCA rows (sample indices) */
  double *evals;           /* [nind]  eigenvalues, descending (nrows valid; K in fastmode) */
  double *evecs;           /* [numeigs*nind] top eigenvectors over the rows, j at j*nrows */
  double *coords;          /* [numeigs*nind] .evec coordinates, sample k of vector j at j*nind+k */
  uint8_t *ind_out;        /* [nind]  1 = sample is written to .evec */
  uint8_t *snp_state;      /* [nsnp]  0 used, 1 pre-filtered, 2 killed by the allele-count rule */
  int32_t *outlier_idx;    /* [nind]  removed samples in removal order (may be NULL) */
  int32_t *outlier_iter;   /* [nind]  outlier-loop pass (1-based) */
  int32_t *outlier_vec;    /* [nind]  eigenvector that flagged it (0-based) */
  double *outlier_score;   /* [nind]  its z-score */
  /* scalar results */
  int32_t nrows, ncols, numeigs, noutliers, npasses;
  double t_phase[8];       /* wall seconds per GP_PH_* phase */
  double gram_flops;       /* algorithmic Gram flops, sum over passes of N_p (N_p+1) M_p */
  double gram_ms;          /* device time of the Gram kernels, sum over passes */
  /* optional (zero-initialise the struct when unused) */
  double *xtx;             /* [nind*nind] or NULL: the last pass's unscaled XTX, nrows x nrows
                              row-major in xindex order (for the GRM dump, smartpca.c:1297) */
  int32_t nused;           /* SNPs in the last pass's Gram (ynumsnps, smartpca.c:1172-1181) */
  double *ffvecs;          /* [numeigs*nsnp] or NULL: the SNP weights of the last pass
                              (ffvecs, smartpca.c:1485-1493), weight j of SNP s (sorted order)
                              at j*nsnp + s, 0 for a SNP the last pass did not use; the
                              writesnpeigs normalisation (:3047-3053) is the caller's */
  uint8_t *snp_lastpass;   /* [nsnp] or NULL: 1 for the columns of the last pass (xsnplist,
                              including SNPs its allele-count rule dropped), else 0 */
  /* the progress lines of the reference's log (smartpca.c:851, :945-946, :1140-1141, :1223,
   * :1264), recorded when pass_stats is set */
  int32_t *pass_stats;     /* [GP_PASS_STATS * (numoutliter + 1)] or NULL: per pass the SNPs its
                              allele-count / missingness rule dropped in that pass (the
                              reference's log prints the running total), the SNPs it used, the
                              samples left by its outlier removal (-1: none removed), and how
                              many dropped SNPs pass_kills lists (at most 10) */
  int32_t *pass_kills;     /* [3 * 10 * (numoutliter + 1)] or NULL (with pass_stats): per pass
                              the first 10 dropped SNPs as (record index, min(n0, n1) clamped at
                              0, missing count) */
  int32_t nodata;          /* SNPs dropped before the passes for at most one valid genotype */
  int32_t nrows0, ncols0;  /* samples and SNPs of the first pass */
} gp_run_result;

#define GP_PASS_STATS 4

void gp_smartpca_defaults(gp_smartpca_opts *o);
int gp_smartpca_run(gp_ctx *ctx, const gp_smartpca_opts *o, const gp_panel *p,
                    gp_run_result *r);

/* set the handle's error text (used by host code layered on the ABI) and return code */
int gp_fail_msg(gp_ctx *ctx, int code, const char *fmt, ...);

/* Tracy-Widom statistics of a spectrum, as smartpca's log prints them
 * (src/eigensrc/smartpca.c:1336-1366; dotwcalc src/nicksrc/statsubs.c:1680-1725): lambda[0..m)
 * the positive eigenvalues of the last pass in descending order (numgtz, > 1e-6), nrows the
 * pass's samples, znval the fixed number of markers (<= 0: estimated per eigenvalue, the
 * default), nostatslim the shortest tail of the spectrum that gets a statistic (smartpca's
 * default 10).  For each i: twstat[i] (Johnstone's normalisation of lambda[i] within
 * lambda[i..m)), pvalue[i] (the right tail of TW1 there, computed on the host; see gp_tw.c)
 * and effn[i] (the effective number of markers); all three -1 where the reference prints NA.
 * Host only; no device is touched. */
int gp_twstats(const double *lambda, int32_t m, int32_t nrows, double znval,
               int32_t nostatslim, double *twstat, double *pvalue, double *effn);
/* the right tail of TW1 at x as smartpca reads it: 1 below -8, the cubic Hermite
 * interpolant of TW1's tail and density on -8.0, -7.9, ..., 8.0 between (statsubs.c:1811-1905),
 * and from 8 on the Margetis-Edelman density (the reference's own value there) */
double gp_tw_tail(double x);
/* the mpstats line (mpestimate, smartpca.c:4532-4560): the 0.25, 0.5 and 0.75 quartiles of
 * lambda[0..m) (linear interpolation of the sorted values at q (m-1)) and (q3 - q1) / q2 in
 * out4; returns 1 (nothing printed by the reference) when m < 10 */
int gp_mpstats(const double *lambda, int32_t m, double *out4);

#ifdef __cplusplus
}
#endif
#endif
