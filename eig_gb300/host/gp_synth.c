/*
 * Seeded Balding–Nichols genotype generator writing packedancestrymap records.
 *
 * Model (the synthetic stand-in for real panels, shapes as in the smartpca workloads):
 *   ancestral p_s        ~ Uniform(p_lo, p_hi)
 *   population freq p_ks ~ Beta(p_s (1-F_k)/F_k, (1-p_s)(1-F_k)/F_k)
 *   admixed sample       p = a p_k1 + (1-a) p_k2 with a ~ Uniform(0,1)
 *   genotype g           ~ Binomial(2, p) = count of the first allele, 0/1/2
 *   missing              with probability miss (per sample miss ~ Uniform(lo,hi) if asked)
 *
 * Packed layout (reference src/mcio.c:2396-2402 header, src/admutils.c:685-735 bit order):
 * a header record of rlen = max(ceil(N/4), 48) bytes holding "GENO %7d %7d %x %x" with the
 * order-dependent string hashes of the sample and SNP IDs (src/admutils.c:651-681), then
 * one rlen-byte record per SNP; sample k sits in byte k>>2 at bits (3-(k&3))*2, MSB first;
 * code 3 = missing.
 *
 * Every genotype is a pure function of (seed, snp, sample), so the output does not depend
 * on the thread count.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gp_synth.h"

/* ---- counter-based randomness ---------------------------------------------------- */

static inline uint64_t mix64(uint64_t z)
{
  /* splitmix64 finaliser (Steele, Lea, Flood 2014) */
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static inline uint64_t key3(uint64_t seed, uint64_t a, uint64_t b, uint64_t c)
{
  return mix64(seed ^ mix64(a * 0xD6E8FEB86659FD93ull ^ mix64(b + 0x632BE59BD9B4E019ull) ^
                            (c << 48)));
}

/* uniform in (0,1) from the top 53 bits */
static inline double u01(uint64_t x)
{
  return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

typedef struct {
  uint64_t state;
} srng;

static inline double srng_u(srng *r)
{
  r->state += 0x9E3779B97F4A7C15ull;
  return u01(mix64(r->state));
}

static double srng_normal(srng *r)
{
  double u1 = srng_u(r), u2 = srng_u(r);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* Gamma(a, 1): Marsaglia & Tsang (2000); a < 1 boosted by U^(1/a). */
static double srng_gamma(srng *r, double a)
{
  if (a < 1.0) {
    double u = srng_u(r);
    return srng_gamma(r, a + 1.0) * pow(u, 1.0 / a);
  }
  double d = a - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  for (;;) {
    double x, v;
    do {
      x = srng_normal(r);
      v = 1.0 + c * x;
    } while (v <= 0.0);
    v = v * v * v;
    double u = srng_u(r);
    if (u < 1.0 - 0.0331 * x * x * x * x) return d * v;
    if (log(u) < 0.5 * x * x + d * (1.0 - v + log(v))) return d * v;
  }
}

static double srng_beta(srng *r, double a, double b)
{
  double x = srng_gamma(r, a), y = srng_gamma(r, b);
  double s = x + y;
  return s > 0.0 ? x / s : 0.5;
}

/* ---- string hashes of the packed header ------------------------------------------ */

int32_t gp_hash_string(const char *s)
{
  /* hashit: h = h*23 + c over the bytes (src/admutils.c:668-681), 32-bit wrap-around */
  uint32_t h = 0;
  for (; *s; ++s) h = h * 23u + (uint32_t)(int32_t)(signed char)*s;
  return (int32_t)h;
}

int32_t gp_hash_list(const char *const *ids, int64_t n)
{
  /* hasharr: h = (h*17) ^ hashit(id) in list order (src/admutils.c:651-666) */
  uint32_t h = 0;
  for (int64_t i = 0; i < n; ++i) {
    h *= 17u;
    h ^= (uint32_t)gp_hash_string(ids[i]);
  }
  return (int32_t)h;
}

int64_t gp_packed_rlen(int32_t nind)
{
  int64_t r = ((int64_t)nind * 2 + 7) / 8;
  return r < 48 ? 48 : r;
}

/* ---- the model --------------------------------------------------------------------- */

typedef struct {
  const gp_synth_spec *spec;
  int32_t *pop_a, *pop_b;   /* per sample: population(s) */
  double *mix;              /* per sample admixture fraction for pop_a */
  double *miss;             /* per sample missing probability */
  uint8_t *records;
  int64_t rlen;
  int64_t snp_lo, snp_hi;
} synth_job;

static void snp_freqs(const gp_synth_spec *sp, int64_t s, double *pk)
{
  srng r = {key3(sp->seed, (uint64_t)s, 0xA5A5ull, 1)};
  double p = sp->p_lo + (sp->p_hi - sp->p_lo) * srng_u(&r);
  for (int k = 0; k < sp->npops; ++k) {
    double F = sp->fst[k];
    if (F <= 0.0) {
      pk[k] = p;
      continue;
    }
    double a = p * (1.0 - F) / F, b = (1.0 - p) * (1.0 - F) / F;
    pk[k] = srng_beta(&r, a, b);
  }
}

/* genotype code of sample n at SNP s given its allele frequency p and missing rate */
static inline int draw_code(uint64_t seed, int64_t s, int64_t n, double p, double miss)
{
  uint64_t h1 = key3(seed, (uint64_t)s, (uint64_t)n, 2);
  uint64_t h2 = mix64(h1 ^ 0x5851F42D4C957F2Dull);
  int g = (u01(h1) < p) + (u01(h2) < p);
  uint64_t h3 = mix64(h2 + 0x14057B7EF767814Full);
  return u01(h3) < miss ? 3 : g;
}

static void *synth_worker(void *arg)
{
  synth_job *job = (synth_job *)arg;
  const gp_synth_spec *sp = job->spec;
  double pk[GP_SYNTH_MAXPOPS];
  for (int64_t s = job->snp_lo; s < job->snp_hi; ++s) {
    snp_freqs(sp, s, pk);
    uint8_t *rec = job->records + s * job->rlen;
    memset(rec, 0, (size_t)job->rlen);
    for (int32_t n = 0; n < sp->nind; ++n) {
      double p = pk[job->pop_a[n]];
      if (job->pop_b[n] >= 0) p = job->mix[n] * p + (1.0 - job->mix[n]) * pk[job->pop_b[n]];
      int g = draw_code(sp->seed, s, n, p, job->miss[n]);
      rec[n >> 2] |= (uint8_t)(g << ((3 - (n & 3)) * 2));
    }
  }
  return NULL;
}

/* ---- new samples of the same populations, in request-row layout ----------------------- */

typedef struct {
  const gp_synth_spec *sp;
  uint64_t sample_seed;
  const int64_t *snp_index;
  int64_t nk, row_bytes;
  double *pk;               /* [nk][npops] */
  int32_t *pop_a, *pop_b;
  double *mix, *miss;
  uint8_t *rows;
  int64_t lo, hi;           /* SNP range (phase 0) or sample range (phase 1) */
  int phase;
} rows_job;

static void *rows_worker(void *arg)
{
  rows_job *j = (rows_job *)arg;
  const gp_synth_spec *sp = j->sp;
  if (j->phase == 0) {
    for (int64_t k = j->lo; k < j->hi; ++k) snp_freqs(sp, j->snp_index[k], j->pk + k * sp->npops);
    return NULL;
  }
  for (int64_t n = j->lo; n < j->hi; ++n) {
    uint8_t *row = j->rows + n * j->row_bytes;
    memset(row, 0xFF, (size_t)j->row_bytes); /* pad codes 3 */
    for (int64_t k = 0; k < j->nk; ++k) {
      const double *pk = j->pk + k * sp->npops;
      double p = pk[j->pop_a[n]];
      if (j->pop_b[n] >= 0) p = j->mix[n] * p + (1.0 - j->mix[n]) * pk[j->pop_b[n]];
      int g = draw_code(j->sample_seed, j->snp_index[k], n, p, j->miss[n]);
      int sh = (3 - (int)(k & 3)) * 2;
      row[k >> 2] = (uint8_t)((row[k >> 2] & ~(3u << sh)) | ((unsigned)g << sh));
    }
  }
  return NULL;
}

static void run_rows_jobs(rows_job *base, int64_t total, int nthreads, int phase)
{
  pthread_t th[256];
  rows_job jobs[256];
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  int64_t per = (total + nthreads - 1) / nthreads;
  int started[256] = {0};
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = *base;
    jobs[t].phase = phase;
    jobs[t].lo = per * t < total ? per * t : total;
    jobs[t].hi = per * (t + 1) < total ? per * (t + 1) : total;
    if (t > 0 && pthread_create(&th[t], NULL, rows_worker, &jobs[t]) == 0) started[t] = 1;
    else if (t > 0) rows_worker(&jobs[t]);
  }
  rows_worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t)
    if (started[t]) pthread_join(th[t], NULL);
}

int gp_synth_sample_rows(const gp_synth_spec *sp, uint64_t sample_seed, const int64_t *snp_index,
                         int64_t nk, int64_t row_bytes, uint8_t *rows, int32_t *pop_of_sample,
                         int nthreads)
{
  if (row_bytes * 4 < nk || nk < 0) return -1;
  gp_synth_spec rs = *sp;
  rs.seed = sample_seed; /* assignment, admixture and missingness of the new samples */
  int32_t *pa = (int32_t *)malloc(sizeof(int32_t) * (size_t)sp->nind);
  int32_t *pb = (int32_t *)malloc(sizeof(int32_t) * (size_t)sp->nind);
  double *mx = (double *)malloc(sizeof(double) * (size_t)sp->nind);
  double *ms = (double *)malloc(sizeof(double) * (size_t)sp->nind);
  double *pk = (double *)malloc(sizeof(double) * (size_t)(nk > 0 ? nk : 1) * sp->npops);
  int rc = 0;
  if (!pa || !pb || !mx || !ms || !pk) {
    rc = -3;
    goto done;
  }
  rc = gp_synth_assign(&rs, pa, pb, mx, ms);
  if (rc) goto done;
  if (pop_of_sample)
    for (int32_t n = 0; n < sp->nind; ++n) pop_of_sample[n] = (pb[n] >= 0) ? sp->npops : pa[n];
  {
    rows_job b = {sp, sample_seed, snp_index, nk, row_bytes, pk, pa, pb, mx, ms, rows, 0, 0, 0};
    run_rows_jobs(&b, nk, nthreads, 0);          /* population frequencies of the panel SNPs */
    run_rows_jobs(&b, sp->nind, nthreads, 1);    /* the samples' rows */
  }
done:
  free(pa);
  free(pb);
  free(mx);
  free(ms);
  free(pk);
  return rc;
}

int gp_synth_assign(const gp_synth_spec *sp, int32_t *pop_a, int32_t *pop_b, double *mix,
                    double *miss)
{
  if (sp->npops < 1 || sp->npops > GP_SYNTH_MAXPOPS) return -1;
  int32_t n = 0;
  for (int k = 0; k < sp->npops; ++k)
    for (int32_t i = 0; i < sp->pop_sizes[k]; ++i, ++n) {
      if (n >= sp->nind) return -2;
      pop_a[n] = k;
      pop_b[n] = -1;
      mix[n] = 1.0;
    }
  for (; n < sp->nind; ++n) {
    /* the remaining samples are two-way admixtures of distinct populations */
    srng r = {key3(sp->seed, 0xFFFFFFFFull, (uint64_t)n, 3)};
    int a = (int)(srng_u(&r) * sp->npops) % sp->npops;
    int b = a;
    if (sp->npops > 1)
      while (b == a) b = (int)(srng_u(&r) * sp->npops) % sp->npops;
    pop_a[n] = a;
    pop_b[n] = (b == a) ? -1 : b;
    mix[n] = srng_u(&r);
  }
  for (n = 0; n < sp->nind; ++n) {
    if (sp->miss_hi > sp->miss_lo) {
      srng r = {key3(sp->seed, 0xFFFFFFFEull, (uint64_t)n, 4)};
      miss[n] = sp->miss_lo + (sp->miss_hi - sp->miss_lo) * srng_u(&r);
    } else {
      miss[n] = sp->miss_lo;
    }
  }
  return 0;
}

int gp_synth_records(const gp_synth_spec *sp, uint8_t *records, int64_t rlen,
                     int32_t *pop_of_sample, int nthreads)
{
  if (rlen < (sp->nind + 3) / 4) return -1;
  int32_t *pa = (int32_t *)malloc(sizeof(int32_t) * (size_t)sp->nind);
  int32_t *pb = (int32_t *)malloc(sizeof(int32_t) * (size_t)sp->nind);
  double *mx = (double *)malloc(sizeof(double) * (size_t)sp->nind);
  double *ms = (double *)malloc(sizeof(double) * (size_t)sp->nind);
  int rc = 0;
  if (!pa || !pb || !mx || !ms) {
    rc = -3;
    goto done;
  }
  rc = gp_synth_assign(sp, pa, pb, mx, ms);
  if (rc) goto done;
  if (pop_of_sample)
    for (int32_t n = 0; n < sp->nind; ++n)
      pop_of_sample[n] = (pb[n] >= 0) ? sp->npops : pa[n]; /* admixed -> extra label */
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  {
    pthread_t th[256];
    synth_job jobs[256];
    int64_t per = (sp->nsnp + nthreads - 1) / nthreads;
    int started = 0;
    for (int t = 0; t < nthreads; ++t) {
      jobs[t].spec = sp;
      jobs[t].pop_a = pa;
      jobs[t].pop_b = pb;
      jobs[t].mix = mx;
      jobs[t].miss = ms;
      jobs[t].records = records;
      jobs[t].rlen = rlen;
      jobs[t].snp_lo = per * t < sp->nsnp ? per * t : sp->nsnp;
      jobs[t].snp_hi = per * (t + 1) < sp->nsnp ? per * (t + 1) : sp->nsnp;
      if (t == 0) continue;
      if (pthread_create(&th[t], NULL, synth_worker, &jobs[t]) == 0) ++started;
      else synth_worker(&jobs[t]);
      (void)started;
    }
    synth_worker(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  }
done:
  free(pa);
  free(pb);
  free(mx);
  free(ms);
  return rc;
}

/* ---- dataset files ------------------------------------------------------------------- */

static void sample_id(char *buf, size_t n, int32_t i) { snprintf(buf, n, "S%07d", i); }
static void snp_id(char *buf, size_t n, int64_t s) { snprintf(buf, n, "rs%09lld", (long long)s); }

int gp_synth_write_dataset(const gp_synth_spec *sp, const char *prefix, int nthreads)
{
  char path[4096], id[64];
  int64_t rlen = gp_packed_rlen(sp->nind);
  uint8_t *rec = (uint8_t *)malloc((size_t)(rlen * sp->nsnp));
  int32_t *pop = (int32_t *)malloc(sizeof(int32_t) * (size_t)sp->nind);
  if (!rec || !pop) {
    free(rec);
    free(pop);
    return -3;
  }
  int rc = gp_synth_records(sp, rec, rlen, pop, nthreads);
  if (rc) goto out;

  /* .ind: ID sex population */
  snprintf(path, sizeof path, "%s.ind", prefix);
  FILE *f = fopen(path, "w");
  if (!f) { rc = -4; goto out; }
  uint32_t ihash = 0;
  for (int32_t i = 0; i < sp->nind; ++i) {
    sample_id(id, sizeof id, i);
    ihash = ihash * 17u ^ (uint32_t)gp_hash_string(id);
    if (pop[i] < sp->npops)
      fprintf(f, "%20s %c %12s%d\n", id, (i & 1) ? 'M' : 'F', "POP", pop[i]);
    else
      fprintf(f, "%20s %c %12s\n", id, (i & 1) ? 'M' : 'F', "ADMIX");
  }
  fclose(f);

  /* .snp: ID chrom genpos(M) physpos ref var; all on chromosome 1, in order */
  snprintf(path, sizeof path, "%s.snp", prefix);
  f = fopen(path, "w");
  if (!f) { rc = -4; goto out; }
  uint32_t shash = 0;
  for (int64_t s = 0; s < sp->nsnp; ++s) {
    snp_id(id, sizeof id, s);
    shash = shash * 17u ^ (uint32_t)gp_hash_string(id);
    fprintf(f, "%20s %3d %14.8f %12lld A G\n", id, 1, (double)(s + 1) * 1e-6,
            (long long)(s + 1) * 1000LL);
  }
  fclose(f);

  /* .geno: header record + SNP records */
  snprintf(path, sizeof path, "%s.geno", prefix);
  f = fopen(path, "wb");
  if (!f) { rc = -4; goto out; }
  {
    char *hdr = (char *)calloc((size_t)rlen + 64, 1);
    snprintf(hdr, (size_t)rlen + 64, "GENO %7d %7lld %x %x", sp->nind, (long long)sp->nsnp,
             ihash, shash);
    fwrite(hdr, 1, (size_t)rlen, f);
    free(hdr);
  }
  fwrite(rec, 1, (size_t)(rlen * sp->nsnp), f);
  fclose(f);
out:
  free(rec);
  free(pop);
  return rc;
}
