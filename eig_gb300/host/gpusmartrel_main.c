/*
 * gpusmartrel -p parfile : the drop-in for the reference `smartrel`
 * (src/eigensrc/smartrel.c main): the smartpca outlier loop on the GPU with smartrel's SNP
 * rule (a SNP whose minor allele count is <= minallelecnt is dropped, :477-480), then the
 * relatedness scan: the top numeigs components are removed from the scaled Gram of the last
 * pass and every pair of samples with normalised residual covariance + 1/(n-1) >= relthresh
 * is printed, highest first (:578-618):
 *
 *   stdout          "rel: %20s %20s  %9.3f\n" per pair; "## nothing above relthresh!" if none
 *   outliername     "REMOVED outlier %s iter %d evec %d sigmage %.3f\n" (:561-563)
 *
 * Parfile keys (smartrel.c:628-750): genotypename snpname indivname poplistname
 * outliername/outlieroutname numoutevec/numeigs numoutlieriter/numoutliter
 * numoutlierevec/numoutleigs outliersigmathresh/outlthresh relthresh minallelecnt
 * usenorm/fancynorm altnormstyle/popgenmode noxdata/xdata numchrom hashcheck familynames, and
 * gpuprecision (FP64 default, SPLIT_FP16, SPLIT_BF16X4, SPLIT_BF16).  Options of the
 * reference that change the matrix (ldregress, missingmode, killr2, fstonly, chrom,
 * popsizelimit, weightname, badsnpname) are refused with an error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gpupca.h"
#include "../../include/gpupca_run.h"
#include "gp_io.h"

static void usage(void) { fprintf(stderr, "usage: gpusmartrel -p parfile\n"); }

static int in_list(const char *pop, char **list, int n)
{
  for (int i = 0; i < n; ++i)
    if (strcmp(pop, list[i]) == 0) return 1;
  return 0;
}

typedef struct {
  int32_t a, b;
  double y;
} rel_pair;

/* highest y first; ties by row order (the reference's sort of -y) */
static int cmp_pair(const void *x, const void *y)
{
  const rel_pair *p = (const rel_pair *)x, *q = (const rel_pair *)y;
  if (p->y > q->y) return -1;
  if (p->y < q->y) return 1;
  if (p->a != q->a) return p->a < q->a ? -1 : 1;
  return p->b < q->b ? -1 : (p->b > q->b);
}

int main(int argc, char **argv)
{
  const char *parname = NULL;
  for (int i = 1; i < argc; ++i)
    if (strcmp(argv[i], "-p") == 0 && i + 1 < argc) parname = argv[++i];
  if (!parname) {
    usage();
    return 1;
  }
  gp_parfile pf;
  if (gp_par_read(parname, &pf) != 0) {
    fprintf(stderr, "cannot read %s\n", parname);
    return 1;
  }
  gp_smartpca_opts o;
  gp_smartpca_defaults(&o);
  const char *genotypename = NULL, *snpname = NULL, *indivname = NULL, *outlierout = NULL,
             *poplistname = NULL, *prec = NULL;
  int32_t familynames = 1, hashcheck = 1, t = 0, minallele = 1;
  double relthresh = 0.05;
  gp_par_str(&pf, "genotypename:", &genotypename);
  gp_par_str(&pf, "snpname:", &snpname);
  gp_par_str(&pf, "indivname:", &indivname);
  gp_par_str(&pf, "poplistname:", &poplistname);
  gp_par_str(&pf, "outliername:", &outlierout);
  gp_par_str(&pf, "outlieroutname:", &outlierout);
  gp_par_str(&pf, "gpuprecision:", &prec);
  gp_par_int(&pf, "numeigs:", &o.numeigs);
  gp_par_int(&pf, "numoutevec:", &o.numeigs);
  gp_par_int(&pf, "numoutliter:", &o.numoutliter);
  gp_par_int(&pf, "numoutlieriter:", &o.numoutliter);
  /* the reference looks this key up without its colon (smartrel.c:725) */
  gp_par_int(&pf, "numoutleigs", &o.numoutleigs);
  gp_par_int(&pf, "numoutlierevec:", &o.numoutleigs);
  gp_par_dbl(&pf, "outlthresh:", &o.outlthresh);
  gp_par_dbl(&pf, "outliersigmathresh:", &o.outlthresh);
  gp_par_dbl(&pf, "relthresh:", &relthresh);
  gp_par_int(&pf, "minallelecnt:", &minallele);
  gp_par_int(&pf, "fancynorm:", &o.fancynorm);
  gp_par_int(&pf, "usenorm:", &o.fancynorm);
  gp_par_int(&pf, "altnormstyle:", &o.altnormstyle);
  gp_par_int(&pf, "popgenmode:", &o.altnormstyle);
  gp_par_int(&pf, "noxdata:", &o.noxdata);
  t = -1;
  if (gp_par_int(&pf, "xdata:", &t) && t >= 0) o.noxdata = 1 - t;
  t = 0;
  gp_par_int(&pf, "numchrom:", &o.numchrom);
  gp_par_int(&pf, "hashcheck:", &hashcheck);
  gp_par_int(&pf, "familynames:", &familynames);
  const char *refuse[] = {"ldregress:", "nsnpldregress:", "missingmode:", "killr2:", "fstonly:",
                          "chrom:", "popsizelimit:"};
  for (size_t i = 0; i < sizeof refuse / sizeof refuse[0]; ++i)
    if (gp_par_int(&pf, refuse[i], &t) && t > 0) {
      fprintf(stderr, "%s is not supported by this path\n", refuse[i]);
      return 1;
    }
  const char *refuse_s[] = {"weightname:", "badsnpname:"};
  for (size_t i = 0; i < sizeof refuse_s / sizeof refuse_s[0]; ++i) {
    const char *v = NULL;
    if (gp_par_str(&pf, refuse_s[i], &v) && v) {
      fprintf(stderr, "%s is not supported by this path\n", refuse_s[i]);
      return 1;
    }
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
  /* smartrel drops a SNP when min(n0, n1) <= minallelecnt and has no missingness limit; the
   * smartpca flow drops it when min < its threshold */
  o.minallelecnt = minallele + 1;
  o.maxmissing = 0x7fffffff;
  o.lsqproject = 0;
  o.fastmode = 0;
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

  const int32_t K = o.numeigs > 0 ? o.numeigs : 1;
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

  gp_ctx *ctx = NULL;
  if (gp_open(0, &ctx)) {
    fprintf(stderr, "gp_open: %s\n", gp_last_error(NULL));
    return 1;
  }
  gp_keep_gram(ctx, 1);
  int rc = gp_smartpca_run(ctx, &o, &p, &r);
  if (rc) {
    fprintf(stderr, "fatalx:\n%s (code %d)\n", gp_last_error(ctx), rc);
    gp_close(ctx);
    return 1;
  }
  printf("number of samples used: %d number of snps used: %d\n", r.nrows, r.ncols);
  FILE *ol = stdout;
  if (outlierout) ol = fopen(outlierout, "w");
  for (int32_t i = 0; i < r.noutliers && ol; ++i)
    fprintf(ol, "REMOVED outlier %s iter %d evec %d sigmage %.3f\n", inds.id[r.outlier_idx[i]],
            r.outlier_iter[i], r.outlier_vec[i], r.outlier_score[i]);
  if (ol && ol != stdout) fclose(ol);

  /* relatedness on the device; grow the output if more pairs pass than fit */
  int64_t cap = 1 << 20, npairs = 0;
  int32_t *pa = NULL, *pb = NULL;
  double *ps = NULL;
  for (;;) {
    pa = (int32_t *)realloc(pa, sizeof(int32_t) * (size_t)cap);
    pb = (int32_t *)realloc(pb, sizeof(int32_t) * (size_t)cap);
    ps = (double *)realloc(ps, sizeof(double) * (size_t)cap);
    if (!pa || !pb || !ps) {
      fprintf(stderr, "no memory for %lld pairs\n", (long long)cap);
      return 1;
    }
    rc = gp_relate(ctx, r.numeigs, relthresh, cap, pa, pb, ps, &npairs);
    if (rc) {
      fprintf(stderr, "gp_relate: %s\n", gp_last_error(ctx));
      return 1;
    }
    if (npairs <= cap) break;
    cap = npairs;
  }
  if (npairs == 0) {
    printf("## nothing above relthresh!\n");
  } else {
    rel_pair *pr = (rel_pair *)malloc(sizeof(rel_pair) * (size_t)npairs);
    for (int64_t i = 0; i < npairs; ++i) {
      pr[i].a = pa[i];
      pr[i].b = pb[i];
      pr[i].y = ps[i];
    }
    qsort(pr, (size_t)npairs, sizeof(rel_pair), cmp_pair);
    for (int64_t i = 0; i < npairs; ++i) {
      printf("rel: %20s ", inds.id[r.xindex[pr[i].a]]);
      printf("%20s ", inds.id[r.xindex[pr[i].b]]);
      printf(" %9.3f\n", pr[i].y);
    }
    free(pr);
  }
  printf("##end of gpusmartrel run\n");
  gp_close(ctx);
  gp_free_snps(&snps);
  gp_free_inds(&inds);
  gp_par_free(&pf);
  free(records);
  return 0;
}
