/*
 * File formats of the smartpca drop-in, host C.
 *   parfile        "key: value" lines, '#' comments, YES/NO ints, upper-case keys substituted
 *                  into other values (openpars/getint/dostrsub src/nicksrc/getpars.c:28-214,
 *                  :378-450)
 *   SNP list       EIGENSTRAT/ANCESTRYMAP .snp "ID chrom genpos physpos [a1 a2]" or PLINK
 *                  .bim/.map "chrom ID genpos physpos" (readsnpdata src/mcio.c:415-600);
 *                  chromosome names X/Y/MT/XY (str2chrom :4545-4572); sorted by (chrom,
 *                  round(genpos*1e6), round(physpos)) as getsnps does (:175-199)
 *   sample list    "ID sex population" with population "Ignore" ignored (readinddata
 *                  :980-1035) or PLINK .fam/.ped first 6 columns (readindpeddata :1040-1135)
 *   genotypes      packedancestrymap with "GENO nind nsnp ihash shash" header record
 *                  (inpack :2769-2865), PLINK .bed (getbedgenos :3893-3992) or EIGENSTRAT
 *                  text, one line of digits per SNP, 9 = missing
 */
#include "gp_io.h"

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gpupca.h"
#include "gp_synth.h"

/* ---- parfile ------------------------------------------------------------------------ */

static char *trim(char *s)
{
  while (*s && isspace((unsigned char)*s)) ++s;
  char *e = s + strlen(s);
  while (e > s && isspace((unsigned char)e[-1])) *--e = 0;
  return s;
}

static int is_upper_key(const char *k)
{
  int any = 0;
  for (; *k && *k != ':'; ++k) {
    if (islower((unsigned char)*k)) return 0;
    if (isupper((unsigned char)*k)) any = 1;
  }
  return any;
}

static char *replace_all(const char *s, const char *from, const char *to)
{
  size_t lf = strlen(from), lt = strlen(to), cnt = 0;
  if (lf == 0) return strdup(s);
  for (const char *p = strstr(s, from); p; p = strstr(p + lf, from)) ++cnt;
  char *out = (char *)malloc(strlen(s) + cnt * (lt + 1) + 1);
  char *o = out;
  const char *p = s;
  for (const char *q = strstr(p, from); q; q = strstr(p, from)) {
    memcpy(o, p, (size_t)(q - p));
    o += q - p;
    memcpy(o, to, lt);
    o += lt;
    p = q + lf;
  }
  strcpy(o, p);
  return out;
}

int gp_par_read(const char *path, gp_parfile *pf)
{
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  char line[4096];
  int cap = 64;
  pf->n = 0;
  pf->key = (char **)malloc(sizeof(char *) * cap);
  pf->val = (char **)malloc(sizeof(char *) * cap);
  while (fgets(line, sizeof line, f)) {
    char *s = trim(line);
    if (!*s || *s == '#') continue;
    char *sp = s;
    while (*sp && !isspace((unsigned char)*sp)) ++sp;
    char *rest = *sp ? sp + 1 : sp;
    *sp = 0;
    char *hash = strchr(rest, '#');
    if (hash) *hash = 0;
    rest = trim(rest);
    if (pf->n == cap) {
      cap *= 2;
      pf->key = (char **)realloc(pf->key, sizeof(char *) * cap);
      pf->val = (char **)realloc(pf->val, sizeof(char *) * cap);
    }
    pf->key[pf->n] = strdup(s);
    pf->val[pf->n] = strdup(rest);
    pf->n++;
  }
  fclose(f);
  /* string substitution of upper-case parameters, longest name first */
  {
    int *order = (int *)malloc(sizeof(int) * (pf->n + 1));
    int nu = 0;
    for (int k = 0; k < pf->n; ++k)
      if (is_upper_key(pf->key[k])) order[nu++] = k;
    /* stable sort by decreasing name length */
    for (int a = 1; a < nu; ++a) {
      int x = order[a], b = a - 1;
      while (b >= 0 && strlen(pf->key[order[b]]) < strlen(pf->key[x])) {
        order[b + 1] = order[b];
        --b;
      }
      order[b + 1] = x;
    }
    for (int u = 0; u < nu; ++u) {
      char name[256];
      snprintf(name, sizeof name, "%s", pf->key[order[u]]);
      size_t l = strlen(name);
      if (l && name[l - 1] == ':') name[l - 1] = 0;
      for (int k = 0; k < pf->n; ++k) {
        if (is_upper_key(pf->key[k])) continue;
        if (!strstr(pf->val[k], name)) continue;
        char *nv = replace_all(pf->val[k], name, pf->val[order[u]]);
        free(pf->val[k]);
        pf->val[k] = nv;
      }
    }
    free(order);
  }
  return 0;
}

void gp_par_free(gp_parfile *pf)
{
  for (int k = 0; k < pf->n; ++k) {
    free(pf->key[k]);
    free(pf->val[k]);
  }
  free(pf->key);
  free(pf->val);
  pf->n = 0;
}

static const char *par_find(const gp_parfile *pf, const char *key)
{
  for (int k = 0; k < pf->n; ++k)
    if (strcmp(pf->key[k], key) == 0) return pf->val[k];
  return NULL;
}

int gp_par_int(const gp_parfile *pf, const char *key, int32_t *out)
{
  const char *v = par_find(pf, key);
  if (!v) return 0;
  char w[256];
  if (sscanf(v, "%255s", w) != 1) return 0;
  if (strcmp(w, "YES") == 0) *out = 1;
  else if (strcmp(w, "NO") == 0) *out = 0;
  else *out = atoi(w);
  return 1;
}

int gp_par_dbl(const gp_parfile *pf, const char *key, double *out)
{
  const char *v = par_find(pf, key);
  if (!v) return 0;
  *out = atof(v);
  return 1;
}

int gp_par_str(const gp_parfile *pf, const char *key, const char **out)
{
  const char *v = par_find(pf, key);
  if (!v) return 0;
  *out = v;
  return 1;
}

/* ---- helpers -------------------------------------------------------------------------- */

static int ends_with(const char *s, const char *suf)
{
  size_t ls = strlen(s), lf = strlen(suf);
  return ls >= lf && strcmp(s + ls - lf, suf) == 0;
}

static int split(char *line, char **tok, int maxtok)
{
  int n = 0;
  char *p = line;
  while (*p && n < maxtok) {
    while (*p && isspace((unsigned char)*p)) ++p;
    if (!*p) break;
    tok[n++] = p;
    while (*p && !isspace((unsigned char)*p)) ++p;
    if (*p) *p++ = 0;
  }
  return n;
}

static int chrom_of(const char *s, int numchrom)
{
  char ss[16];
  if (strncmp(s, "chr", 3) == 0) s += 3;
  snprintf(ss, sizeof ss, "%s", s);
  for (char *p = ss; *p; ++p) *p = (char)toupper((unsigned char)*p);
  if (strcmp(ss, "X") == 0) return numchrom + 1;
  if (strcmp(ss, "Y") == 0) return numchrom + 2;
  if (strcmp(ss, "MT") == 0) return 90;
  if (strcmp(ss, "XY") == 0) return 91;
  if (strcmp(ss, "2A") == 0 || strcmp(ss, "2B") == 0) return 2;
  for (char *p = ss; *p; ++p)
    if (!isdigit((unsigned char)*p)) return -1;
  return atoi(ss);
}

static long long nnint(double x) { return (long long)(x < 0 ? x - 0.5 : x + 0.5); }

/* ---- SNP list ------------------------------------------------------------------------- */

static const gp_snplist *g_sort_snps;

static int snp_cmp(const void *a, const void *b)
{
  int64_t i = *(const int64_t *)a, j = *(const int64_t *)b;
  const gp_snplist *s = g_sort_snps;
  if (s->chrom[i] != s->chrom[j]) return s->chrom[i] < s->chrom[j] ? -1 : 1;
  long long gi = nnint(s->gpos[i] * 1e6), gj = nnint(s->gpos[j] * 1e6);
  if (gi != gj) return gi < gj ? -1 : 1;
  long long pi = nnint(s->ppos[i]), pj = nnint(s->ppos[j]);
  if (pi != pj) return pi < pj ? -1 : 1;
  return i < j ? -1 : (i > j);
}

int gp_read_snps(const char *path, int numchrom, gp_snplist *s, char *err, int errlen)
{
  FILE *f = fopen(path, "r");
  if (!f) {
    snprintf(err, errlen, "cannot open SNP file %s", path);
    return -1;
  }
  int plink = ends_with(path, ".bim") || ends_with(path, ".map") || ends_with(path, ".pedsnp");
  int64_t cap = 1024;
  memset(s, 0, sizeof *s);
  s->id = malloc(sizeof(*s->id) * cap);
  s->chrom = malloc(sizeof(int32_t) * cap);
  s->gpos = malloc(sizeof(double) * cap);
  s->ppos = malloc(sizeof(double) * cap);
  s->alleles = malloc(sizeof(*s->alleles) * cap);
  char line[4096], *tok[16];
  while (fgets(line, sizeof line, f)) {
    int nt = split(line, tok, 16);
    if (nt == 0 || tok[0][0] == '#') continue;
    if (nt < 4) {
      snprintf(err, errlen, "bad SNP line in %s", path);
      fclose(f);
      return -1;
    }
    if (s->n == cap) {
      cap *= 2;
      s->id = realloc(s->id, sizeof(*s->id) * cap);
      s->chrom = realloc(s->chrom, sizeof(int32_t) * cap);
      s->gpos = realloc(s->gpos, sizeof(double) * cap);
      s->ppos = realloc(s->ppos, sizeof(double) * cap);
      s->alleles = realloc(s->alleles, sizeof(*s->alleles) * cap);
    }
    const char *id = plink ? tok[1] : tok[0];
    const char *ch = plink ? tok[0] : tok[1];
    snprintf(s->id[s->n], GP_IDLEN, "%s", id);
    s->chrom[s->n] = chrom_of(ch, numchrom);
    s->gpos[s->n] = atof(tok[2]);
    s->ppos[s->n] = atof(tok[3]);
    /* alleles: upper-cased first characters of columns 5 and 6 (readsnpdata,
     * src/mcio.c:509-514); in a PLINK map as they are, '0' read as 'X' (readsnpmapdata
     * :571-585) */
    s->alleles[s->n][0] = s->alleles[s->n][1] = 0;
    if (nt >= 6) {
      for (int a = 0; a < 2; ++a) {
        char c = tok[4 + a][0];
        if (plink)
          c = c == '0' ? 'X' : c;
        else
          c = (char)toupper((unsigned char)c);
        s->alleles[s->n][a] = c;
      }
    }
    s->n++;
  }
  fclose(f);
  /* genetic positions (src/mcio.c:517-535): all zero -> 1e-8 * physical position; else, if
   * any exceeds 100, they are centimorgans and become morgans */
  double maxg = -9999.0;
  int usecm = 0;
  for (int64_t i = 0; i < s->n; ++i) {
    if (s->gpos[i] > maxg) maxg = s->gpos[i];
    if (s->gpos[i] > 100) usecm = 1;
  }
  if (s->n > 0 && maxg <= 0.00001) {
    for (int64_t i = 0; i < s->n; ++i) s->gpos[i] = 1.0e-8 * s->ppos[i];
  } else if (usecm) {
    for (int64_t i = 0; i < s->n; ++i) s->gpos[i] /= 100.0;
  }
  s->order = malloc(sizeof(int64_t) * (s->n ? s->n : 1));
  for (int64_t i = 0; i < s->n; ++i) s->order[i] = i;
  g_sort_snps = s;
  qsort(s->order, (size_t)s->n, sizeof(int64_t), snp_cmp);
  return 0;
}

void gp_free_snps(gp_snplist *s)
{
  free(s->id);
  free(s->chrom);
  free(s->gpos);
  free(s->ppos);
  free(s->alleles);
  free(s->order);
  memset(s, 0, sizeof *s);
}

/* ---- sample list ---------------------------------------------------------------------- */

int gp_read_inds(const char *path, int familynames, gp_indlist *ind, char *err, int errlen)
{
  FILE *f = fopen(path, "r");
  if (!f) {
    snprintf(err, errlen, "cannot open sample file %s", path);
    return -1;
  }
  int ped = ends_with(path, ".fam") || ends_with(path, ".ped") || ends_with(path, ".pedind");
  int32_t cap = 256;
  memset(ind, 0, sizeof *ind);
  ind->id = malloc(sizeof(*ind->id) * cap);
  ind->pop = malloc(sizeof(*ind->pop) * cap);
  ind->gender = malloc((size_t)cap);
  ind->ignore = malloc((size_t)cap);
  static char line[1 << 20];
  char *tok[8];
  while (fgets(line, sizeof line, f)) {
    int nt = split(line, tok, 8);
    if (nt == 0 || tok[0][0] == '#') continue;
    if ((!ped && nt < 3) || (ped && nt < 6)) {
      snprintf(err, errlen, "bad sample line in %s", path);
      fclose(f);
      return -1;
    }
    if (ind->n == cap) {
      cap *= 2;
      ind->id = realloc(ind->id, sizeof(*ind->id) * cap);
      ind->pop = realloc(ind->pop, sizeof(*ind->pop) * cap);
      ind->gender = realloc(ind->gender, (size_t)cap);
      ind->ignore = realloc(ind->ignore, (size_t)cap);
    }
    int32_t k = ind->n;
    ind->ignore[k] = 0;
    if (!ped) {
      snprintf(ind->id[k], GP_IDLEN, "%s", tok[0]);
      ind->gender[k] = tok[1][0];
      snprintf(ind->pop[k], GP_IDLEN, "%s", tok[2]);
      if (strcmp(tok[2], "Ignore") == 0) ind->ignore[k] = 1;
    } else {
      if (familynames)
        snprintf(ind->id[k], GP_IDLEN, "%s:%s", tok[0], tok[1]);
      else
        snprintf(ind->id[k], GP_IDLEN, "%s", tok[1]);
      int sx = atoi(tok[4]);
      ind->gender[k] = sx == 1 ? 'M' : sx == 2 ? 'F' : 'U';
      const char *ph = tok[5];
      if (!strcmp(ph, "-9") || !strcmp(ph, "9") || !strcmp(ph, "0")) {
        ind->ignore[k] = 1;
        snprintf(ind->pop[k], GP_IDLEN, "%s", "Ignore");
      } else if (!strcmp(ph, "1")) {
        snprintf(ind->pop[k], GP_IDLEN, "%s", "Control");
      } else if (!strcmp(ph, "2")) {
        snprintf(ind->pop[k], GP_IDLEN, "%s", "Case");
      } else {
        snprintf(ind->pop[k], GP_IDLEN, "%s", ph);
      }
    }
    ind->n++;
  }
  fclose(f);
  return 0;
}

void gp_free_inds(gp_indlist *ind)
{
  free(ind->id);
  free(ind->pop);
  free(ind->gender);
  free(ind->ignore);
  memset(ind, 0, sizeof *ind);
}

/* ---- genotypes ------------------------------------------------------------------------ */

int gp_read_genotypes(const char *path, const gp_snplist *s, const gp_indlist *ind,
                      int hashcheck, uint8_t **out_records, int64_t *rec_bytes, int32_t *code,
                      char *err, int errlen)
{
  FILE *f = fopen(path, "rb");
  if (!f) {
    snprintf(err, errlen, "cannot open genotype file %s", path);
    return -1;
  }
  const int32_t N = ind->n;
  const int64_t M = s->n;
  unsigned char head[48];
  size_t got = fread(head, 1, sizeof head, f);
  uint8_t *in = NULL;
  int64_t rlen = 0;
  int is_bed = got >= 3 && head[0] == 0x6C && head[1] == 0x1B && head[2] == 0x01;
  int is_packed = got >= 4 && memcmp(head, "GENO", 4) == 0;
  if (is_bed || is_packed) {
    rlen = is_bed ? ((int64_t)N + 3) / 4 : gp_packed_rlen(N);
    int64_t off = is_bed ? 3 : rlen;
    if (is_packed) {
      int xn = 0, xs = 0;
      unsigned int ih = 0, sh = 0;
      char hb[256];
      fseek(f, 0, SEEK_SET);
      size_t hl = fread(hb, 1, rlen < 255 ? (size_t)rlen : 255, f);
      hb[hl] = 0;
      if (sscanf(hb, "GENO %d %d %x %x", &xn, &xs, &ih, &sh) != 4) {
        snprintf(err, errlen, "bad packed header in %s", path);
        fclose(f);
        return -1;
      }
      if (xn != N || xs != M) {
        snprintf(err, errlen, "number of samples/SNPs %d/%d != %d/%lld in %s", xn, xs, N,
                 (long long)M, path);
        fclose(f);
        return -1;
      }
      if (hashcheck) {
        uint32_t h = 0;
        for (int32_t k = 0; k < N; ++k) h = h * 17u ^ (uint32_t)gp_hash_string(ind->id[k]);
        if (h != ih) {
          snprintf(err, errlen, "sample file has changed since genotype file was created");
          fclose(f);
          return -1;
        }
        h = 0;
        for (int64_t i = 0; i < M; ++i) h = h * 17u ^ (uint32_t)gp_hash_string(s->id[s->order[i]]);
        if (h != sh) {
          snprintf(err, errlen, "SNP file has changed since genotype file was created");
          fclose(f);
          return -1;
        }
      }
    }
    in = (uint8_t *)malloc((size_t)(rlen * M));
    if (!in) {
      fclose(f);
      snprintf(err, errlen, "out of memory");
      return -1;
    }
    fseek(f, (long)off, SEEK_SET);
    size_t want = (size_t)(rlen * M), r = fread(in, 1, want, f);
    fclose(f);
    if (r != want) {
      free(in);
      snprintf(err, errlen, "genotype file %s is short (%zu of %zu bytes)", path, r, want);
      return -1;
    }
    *code = is_bed ? GP_CODE_BED : GP_CODE_PACKED;
  } else {
    /* EIGENSTRAT text: line i = SNP i (input order), one digit per sample, 9 missing */
    fseek(f, 0, SEEK_SET);
    rlen = gp_packed_rlen(N);
    in = (uint8_t *)calloc((size_t)(rlen * M), 1);
    char *line = (char *)malloc((size_t)N + 64);
    for (int64_t i = 0; i < M; ++i) {
      if (!fgets(line, N + 64, f)) {
        snprintf(err, errlen, "genotype file %s has fewer lines than SNPs", path);
        free(line);
        free(in);
        fclose(f);
        return -1;
      }
      uint8_t *rec = in + i * rlen;
      for (int32_t k = 0; k < N; ++k) {
        int c = line[k];
        int g = (c >= '0' && c <= '2') ? c - '0' : 3;
        rec[k >> 2] |= (uint8_t)(g << ((3 - (k & 3)) * 2));
      }
      for (int32_t k = N; k < rlen * 4; ++k) rec[k >> 2] |= (uint8_t)(3 << ((3 - (k & 3)) * 2));
    }
    free(line);
    fclose(f);
    *code = GP_CODE_PACKED;
  }
  /* records in sorted SNP order */
  uint8_t *out = (uint8_t *)malloc((size_t)(rlen * M));
  if (!out) {
    free(in);
    snprintf(err, errlen, "out of memory");
    return -1;
  }
  for (int64_t i = 0; i < M; ++i) memcpy(out + i * rlen, in + s->order[i] * rlen, (size_t)rlen);
  free(in);
  *out_records = out;
  *rec_bytes = rlen;
  return 0;
}

/* ---- GRM dump ----------------------------------------------------------------------- */

int gp_write_grm(const char *name, int binary, const double *xtx, int32_t n, int32_t numsnps,
                 char (*ids)[GP_IDLEN], const int32_t *xindex, char *err, int errlen)
{
  char path[4096];
  snprintf(path, sizeof path, "%s.id", name);
  FILE *f = fopen(path, "w");
  if (!f) {
    snprintf(err, (size_t)errlen, "cannot write %s", path);
    return -1;
  }
  for (int32_t a = 0; a < n; ++a) fprintf(f, "%s\t%s\n", "NA", ids[xindex[a]]);
  fclose(f);
  /* the PCA's scaling, with the reference's operation order: trace as a running sum of the
   * diagonal, then XTX *= 1/y with y = trace/(n-1) */
  double tr = 0.0;
  for (int32_t a = 0; a < n; ++a) tr += xtx[(size_t)a * n + a];
  const double ys = 1.0 / (tr / (double)(n - 1));
  if (binary) {
    snprintf(path, sizeof path, "%s.N.bin", name);
    f = fopen(path, "wb");
    if (!f) {
      snprintf(err, (size_t)errlen, "cannot write %s", path);
      return -1;
    }
    int32_t w = numsnps;
    const int64_t nout = (int64_t)n * (n + 1) / 2;
    for (int64_t i = 0; i < nout; ++i) fwrite(&w, 4, 1, f);
    fclose(f);
    double ts = 0.0;
    for (int32_t a = 0; a < n; ++a) ts += xtx[(size_t)a * n + a] * ys;
    const double ynorm = ts / (double)n;
    snprintf(path, sizeof path, "%s.bin", name);
    f = fopen(path, "wb");
    if (!f) {
      snprintf(err, (size_t)errlen, "cannot write %s", path);
      return -1;
    }
    for (int32_t a = 0; a < n; ++a)
      for (int32_t b = 0; b <= a; ++b) {
        float y = (float)(xtx[(size_t)a * n + b] * ys / ynorm);
        fwrite(&y, 4, 1, f);
      }
    fclose(f);
    return 0;
  }
  double ds = 0.0;
  for (int32_t a = 0; a < n; ++a) ds += xtx[(size_t)a * n + a] * ys;
  const double recip = (double)n / ds;
  f = fopen(name, "w");
  if (!f) {
    snprintf(err, (size_t)errlen, "cannot write %s", name);
    return -1;
  }
  for (int32_t a = 0; a < n; ++a)
    for (int32_t b = 0; b <= a; ++b) {
      fprintf(f, "%d %d ", a + 1, b + 1);
      fprintf(f, "%d ", numsnps);
      fprintf(f, "%0.6f\n", xtx[(size_t)a * n + b] * ys * recip);
    }
  fclose(f);
  return 0;
}
