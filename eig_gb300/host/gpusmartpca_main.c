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
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "../../include/gpupca.h"
#include "../../include/gpupca_run.h"
#include "gp_io.h"

static void usage(void) { fprintf(stderr, "usage: gpusmartpca -p parfile\n"); }

static int in_list(const char *pop, char **list, int n)
{
  for (int i = 0; i < n; ++i)
    if (strcmp(pop, list[i]) == 0) return 1;
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
             *grmout = NULL;
  int32_t hiprec = 0, familynames = 1, hashcheck = 1, t = 0, xdata = -1, seed = 0,
          grmbinary = 0;
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
  gp_par_int(&pf, "grmbinary:", &grmbinary);
  gp_par_int(&pf, "numeigs:", &o.numeigs);
  gp_par_int(&pf, "numoutevec:", &o.numeigs);
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
  if (gp_par_int(&pf, "missingmode:", &t) && t) {
    fprintf(stderr, "missingmode: YES is not supported by this path\n");
    return 1;
  }
  if (gp_par_int(&pf, "usepopsformissing:", &t) && t) {
    fprintf(stderr, "usepopsformissing: YES is not supported by this path\n");
    return 1;
  }
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
  if (grmout && !o.fastmode) {
    r.xtx = (double *)malloc(sizeof(double) * (size_t)N * N);
    if (!r.xtx) {
      fprintf(stderr, "no memory for the GRM (%d samples)\n", N);
      return 1;
    }
  }

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
  printf("number of samples used: %d number of snps used: %d\n", r.nrows, r.ncols);
  printf("passes: %d  outliers removed: %d\n", r.npasses, r.noutliers);

  FILE *ol = stdout;
  if (outlierout) ol = fopen(outlierout, "w");
  for (int32_t i = 0; i < r.noutliers && ol; ++i) {
    int32_t k = r.outlier_idx[i];
    fprintf(ol, "REMOVED outlier %s iter %d evec %d sigmage %.3f pop: %s\n", inds.id[k],
            r.outlier_iter[i], r.outlier_vec[i], r.outlier_score[i], inds.pop[k]);
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
