/*
 * gpuconvertf -p parfile : the drop-in for the reference `convertf` (src/convertf.c main)
 * on its default path, with the genotype records encoded on the GPU (gp_encode_records).
 *
 * Input: packedancestrymap, PLINK bed/bim/fam or EIGENSTRAT text (genotypename snpname
 * indivname).  Output (outputformat: PACKEDANCESTRYMAP, PACKEDPED or EIGENSTRAT;
 * genotypeoutname snpoutname indivoutname), with the reference's rules on the way:
 *
 *   - SNPs outside chromosomes minchrom..maxchrom (1..97), or outside chrom:/lopos:/hipos:
 *     when chrom: is set, are dropped (convertf.c:288-310);
 *   - samples of population "Ignore" are dropped; with poplistname only the listed
 *     populations are kept (:446-455);
 *   - deletedup (default YES): of consecutive SNPs at one chromosome position only the one
 *     with the shorter ID (equal lengths: the larger ID) is kept (dedupit/pickx :881-943);
 *   - a SNP whose first allele is 0/X/N/D/I and second allele is not is flipped: alleles
 *     swapped and each observed genotype g written as 2 - g (:356-368, flip1 :1017-1026);
 *   - samples with no observed genotype on the kept SNPs are dropped (:476-487).
 *
 * Files written as outfiles (src/mcio.c:3206-3258) does: .snp lines "%20s %5s " + genetic
 * position ("%15.0f" when 0, else "%15.6f") + " %15.0f" physical position + " %c" per allele
 * (printsnps :1931-2015); .ind lines "%20s %c %10s" (printdata :2031-2121); .bim lines
 * "%-2s %12s %12.6f %12.0f" + alleles (printmap :3786-3811); .fam lines "%6d   %12s 0 0 %d %d"
 * (outindped :3449-3499); the GENO header record "GENO %7d %7d %x %x" with the hashes of
 * the written sample and SNP IDs (outpack :2343-2420); the bed magic 6c 1b 01.
 *
 * Options that change the data in other ways (badsnpname, flipsnpname, flipstrandname,
 * polarize, usesamples, newsnpname, newindivname, mkdiploid, killr2, hwfilter, xregionname,
 * fastdup, decimate, downsample, maxmissing, maxmissfrac, minvalpop,
 * fillmissingpoplistname, outputall, outputgroup, familypopnames, sevencolumnped,
 * phasedmode) and the unpacked ANCESTRYMAP/PED outputs are refused with an error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gpupca.h"
#include "gp_io.h"
#include "gp_synth.h"

static void usage(void) { fprintf(stderr, "usage: gpuconvertf -p parfile\n"); }

/* pedval (src/mcio.c:3848-3887) modulo 5: 0 for an unknown allele */
static int allele_ok(char c)
{
  switch (c) {
  case 'A': case 'C': case 'G': case 'T': case '1': case '2': case '3': case '4':
    return 1;
  case 'X': case 'N': case 'D': case 'I': case '0':
    return 0;
  default:
    return 4; /* 9 % 5 */
  }
}

static int fail(const char *msg, const char *arg)
{
  fprintf(stderr, "fatalx:\n%s%s\n", msg, arg ? arg : "");
  return 1;
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
  if (gp_par_read(parname, &pf) != 0) return fail("cannot read ", parname);
  const char *genotypename = NULL, *snpname = NULL, *indivname = NULL, *poplistname = NULL;
  const char *gout = NULL, *sout = NULL, *iout = NULL, *omode = "PACKEDANCESTRYMAP";
  int32_t familynames = 1, hashcheck = 1, numchrom = 22, minchrom = 1, maxchrom = 97;
  int32_t xchrom = -1, lopos = -999999999, hipos = 999999999, deletedup = 1, t = 0;
  gp_par_str(&pf, "genotypename:", &genotypename);
  gp_par_str(&pf, "snpname:", &snpname);
  gp_par_str(&pf, "indivname:", &indivname);
  gp_par_str(&pf, "poplistname:", &poplistname);
  gp_par_str(&pf, "genooutfilename:", &gout);
  gp_par_str(&pf, "genotypeoutname:", &gout);
  gp_par_str(&pf, "snpoutfilename:", &sout);
  gp_par_str(&pf, "snpoutname:", &sout);
  gp_par_str(&pf, "indoutfilename:", &iout);
  gp_par_str(&pf, "indivoutname:", &iout);
  gp_par_str(&pf, "outputformat:", &omode);
  gp_par_str(&pf, "outputmode:", &omode);
  gp_par_int(&pf, "familynames:", &familynames);
  gp_par_int(&pf, "hashcheck:", &hashcheck);
  gp_par_int(&pf, "numchrom:", &numchrom);
  gp_par_int(&pf, "minchrom:", &minchrom);
  gp_par_int(&pf, "maxchrom:", &maxchrom);
  gp_par_int(&pf, "chrom:", &xchrom);
  gp_par_int(&pf, "lopos:", &lopos);
  gp_par_int(&pf, "hipos:", &hipos);
  gp_par_int(&pf, "deletedup:", &deletedup);
  const char *refuse_s[] = {"badsnpname:", "flipsnpname:", "flipstrandname:", "polarize:",
                            "usesamples:", "newsnpname:", "newindivname:", "xregionname:",
                            "fillmissingpoplistname:", "genotypelist:"};
  for (size_t i = 0; i < sizeof refuse_s / sizeof refuse_s[0]; ++i) {
    const char *v = NULL;
    if (gp_par_str(&pf, refuse_s[i], &v) && v)
      return fail("not supported by this path: ", refuse_s[i]);
  }
  const char *refuse_i[] = {"mkdiploid:", "killr2:", "fastdup:", "decimate:", "downsample:",
                            "maxmissing:", "minvalpop:", "outputall:", "outputgroup:",
                            "familypopnames:", "sevencolumnped:", "phasedmode:", "chimpmode:"};
  for (size_t i = 0; i < sizeof refuse_i / sizeof refuse_i[0]; ++i)
    if (gp_par_int(&pf, refuse_i[i], &t) && t > 0)
      return fail("not supported by this path: ", refuse_i[i]);
  double dv = -1.0;
  if ((gp_par_dbl(&pf, "hwfilter:", &dv) && dv > 0) ||
      (gp_par_dbl(&pf, "r2thresh:", &dv) && dv > 0))
    return fail("not supported by this path: ", "hwfilter / r2thresh");
  if (gp_par_dbl(&pf, "maxmissfrac:", &dv) && dv < 1.0)
    return fail("not supported by this path: ", "maxmissfrac");
  int32_t format;
  if (strcmp(omode, "PACKEDANCESTRYMAP") == 0) format = GP_OUT_PACKEDANCESTRYMAP;
  else if (strcmp(omode, "PACKEDPED") == 0) format = GP_OUT_PACKEDPED;
  else if (strcmp(omode, "EIGENSTRAT") == 0) format = GP_OUT_EIGENSTRAT;
  else return fail("outputformat not supported by this path: ", omode);
  if (!genotypename || !snpname || !indivname)
    return fail("genotypename, snpname and indivname are required", NULL);

  char err[512];
  gp_snplist snps;
  gp_indlist inds;
  if (gp_read_snps(snpname, numchrom, &snps, err, sizeof err) ||
      gp_read_inds(indivname, familynames, &inds, err, sizeof err))
    return fail(err, NULL);
  uint8_t *records = NULL;
  int64_t rb = 0;
  int32_t code = 0;
  if (gp_read_genotypes(genotypename, &snps, &inds, hashcheck, &records, &rb, &code, err,
                        sizeof err))
    return fail(err, NULL);
  const int64_t M = snps.n;
  const int32_t N = inds.n;
  /* per sorted SNP: ignore flag and flip */
  uint8_t *ign = (uint8_t *)calloc((size_t)M + 1, 1), *flip = (uint8_t *)calloc((size_t)M + 1, 1);
  for (int64_t i = 0; i < M; ++i) {
    const int64_t r = snps.order[i];
    const int c = snps.chrom[r];
    if (c <= 0 || c > maxchrom || c < minchrom) ign[i] = 1;
    if (xchrom > 0) {
      const double p = snps.ppos[r];
      const long long ip = (long long)(p < 0 ? p - 0.5 : p + 0.5);
      if (c != xchrom || ip < lopos || ip > hipos) ign[i] = 1;
    }
  }
  if (deletedup) {
    int64_t prev = -1;
    for (int64_t i = 0; i < M; ++i) {
      if (ign[i]) continue;
      const int64_t r = snps.order[i];
      if (prev < 0 || snps.chrom[snps.order[prev]] != snps.chrom[r] ||
          snps.ppos[snps.order[prev]] != snps.ppos[r]) {
        prev = i;
        continue;
      }
      const char *a = snps.id[snps.order[prev]], *b = snps.id[r];
      const size_t la = strlen(a), lb = strlen(b);
      int keep_prev = la < lb ? 1 : (lb < la ? 0 : strcmp(a, b) >= 0);
      if (keep_prev) {
        ign[i] = 1;
      } else {
        ign[prev] = 1;
        prev = i;
      }
    }
  }
  int64_t nflip = 0;
  for (int64_t i = 0; i < M; ++i) {
    char *al = snps.alleles[snps.order[i]];
    if (allele_ok(al[0]) == 0 && allele_ok(al[1]) > 0) {
      const char c = al[0];
      al[0] = al[1];
      al[1] = c;
      flip[i] = 1;
      ++nflip;
    }
  }
  /* samples */
  uint8_t *keep = (uint8_t *)calloc((size_t)N + 1, 1), *aff = (uint8_t *)calloc((size_t)N + 1, 1);
  char **plist = NULL;
  int np = 0;
  if (poplistname) {
    FILE *pl = fopen(poplistname, "r");
    if (!pl) return fail("cannot open ", poplistname);
    char line[1024];
    plist = (char **)malloc(sizeof(char *) * 65536);
    while (fgets(line, sizeof line, pl) && np < 65536) {
      char w[256];
      if (sscanf(line, "%255s", w) != 1 || w[0] == '#') continue;
      plist[np++] = strdup(w);
    }
    fclose(pl);
  }
  for (int32_t k = 0; k < N; ++k) {
    keep[k] = !inds.ignore[k];
    if (poplistname) {
      int in = 0;
      for (int j = 0; j < np && !in; ++j) in = strcmp(inds.pop[k], plist[j]) == 0;
      aff[k] = (uint8_t)in;
      if (!in) keep[k] = 0;
    } else {
      aff[k] = strcmp(inds.pop[k], "Case") == 0;
    }
  }
  int64_t nkeep_snp = 0;
  for (int64_t i = 0; i < M; ++i) nkeep_snp += !ign[i];
  if (nkeep_snp == 0) return fail("no valid snps", NULL);

  gp_ctx *ctx = NULL;
  if (gp_open(0, &ctx)) return fail("gp_open: ", gp_last_error(NULL));
  if (gp_load_genotypes(ctx, records, rb, M, N, code)) return fail(gp_last_error(ctx), NULL);
  free(records);
  /* samples with no observed genotype on the kept SNPs */
  uint8_t *snp_use = (uint8_t *)malloc((size_t)M + 1);
  for (int64_t i = 0; i < M; ++i) snp_use[i] = !ign[i];
  int32_t *svalid = (int32_t *)calloc((size_t)N + 1, sizeof(int32_t));
  if (gp_valid_counts(ctx, NULL, snp_use, NULL, svalid)) return fail(gp_last_error(ctx), NULL);
  int32_t nout = 0;
  for (int32_t k = 0; k < N; ++k) {
    if (keep[k] && svalid[k] == 0) {
      keep[k] = 0;
      printf("no data for individual: %s\n", inds.id[k]);
    }
    nout += keep[k];
  }
  if (nout == 0) return fail("no valid samples!", NULL);
  int32_t *sidx = (int32_t *)malloc(sizeof(int32_t) * (size_t)nout);
  for (int32_t k = 0, j = 0; k < N; ++k)
    if (keep[k]) sidx[j++] = k;
  int64_t *sel = (int64_t *)malloc(sizeof(int64_t) * (size_t)nkeep_snp);
  uint8_t *sflip = (uint8_t *)malloc((size_t)nkeep_snp);
  for (int64_t i = 0, j = 0; i < M; ++i)
    if (!ign[i]) {
      sflip[j] = flip[i];
      sel[j++] = i;
    }
  printf("numvalidind:  %5d  snps: %lld  flipped: %lld\n", nout, (long long)nkeep_snp,
         (long long)nflip);

  /* SNP and sample files */
  if (sout && strcmp(sout, "NULL") != 0) {
    FILE *f = fopen(sout, "w");
    if (!f) return fail("cannot write ", sout);
    for (int64_t j = 0; j < nkeep_snp; ++j) {
      const int64_t r = snps.order[sel[j]];
      char cs[16];
      snprintf(cs, sizeof cs, "%d", snps.chrom[r]);
      if (format == GP_OUT_PACKEDPED) {
        fprintf(f, "%-2s", cs);
        fprintf(f, " %12s", snps.id[r]);
        fprintf(f, " %12.6f", snps.gpos[r]);
        fprintf(f, " %12.0f", snps.ppos[r]);
      } else {
        fprintf(f, "%20s %5s ", snps.id[r], cs);
        if (snps.gpos[r] == 0.0)
          fprintf(f, "%15.0f %15.0f", snps.gpos[r], snps.ppos[r]);
        else
          fprintf(f, "%15.6f %15.0f", snps.gpos[r], snps.ppos[r]);
      }
      for (int a = 0; a < 2; ++a)
        if (snps.alleles[r][a]) fprintf(f, " %c", snps.alleles[r][a]);
      fprintf(f, "\n");
    }
    fclose(f);
  }
  if (iout && strcmp(iout, "NULL") != 0) {
    FILE *f = fopen(iout, "w");
    if (!f) return fail("cannot write ", iout);
    for (int32_t j = 0; j < nout; ++j) {
      const int32_t k = sidx[j];
      if (format == GP_OUT_PACKEDPED) {
        const char g = inds.gender[k];
        fprintf(f, "%6d ", j + 1);
        fprintf(f, "  %12s", inds.id[k]);
        fprintf(f, " %d %d", 0, 0);
        fprintf(f, " %d", g == 'M' ? 1 : (g == 'F' ? 2 : 0));
        fprintf(f, " %d", aff[k] + 1);
        fprintf(f, "\n");
      } else {
        fprintf(f, "%20s %c %10s", inds.id[k], inds.gender[k], inds.pop[k]);
        fprintf(f, "\n");
      }
    }
    fclose(f);
  }
  /* genotype file: header, then records encoded on the device in chunks */
  if (gout && strcmp(gout, "NULL") != 0) {
    FILE *f = fopen(gout, "wb");
    if (!f) return fail("cannot write ", gout);
    const int64_t orb = gp_record_bytes(format, nout);
    if (format == GP_OUT_PACKEDANCESTRYMAP) {
      const char **ids = (const char **)malloc(sizeof(char *) * (size_t)(nout > nkeep_snp ? nout : nkeep_snp));
      for (int32_t j = 0; j < nout; ++j) ids[j] = inds.id[sidx[j]];
      const int32_t ih = gp_hash_list(ids, nout);
      for (int64_t j = 0; j < nkeep_snp; ++j) ids[j] = snps.id[snps.order[sel[j]]];
      const int32_t sh = gp_hash_list(ids, nkeep_snp);
      free(ids);
      char *head = (char *)calloc((size_t)orb + 64, 1);
      snprintf(head, (size_t)orb + 64, "GENO %7d %7lld %x %x", nout, (long long)nkeep_snp,
               (unsigned)ih, (unsigned)sh);
      fwrite(head, 1, (size_t)orb, f);
      free(head);
    } else if (format == GP_OUT_PACKEDPED) {
      const unsigned char magic[3] = {0x6C, 0x1B, 0x01};
      fwrite(magic, 1, 3, f);
    }
    int64_t chunk = ((int64_t)256 << 20) / orb;
    if (chunk < 1) chunk = 1;
    if (chunk > nkeep_snp) chunk = nkeep_snp;
    uint8_t *buf = (uint8_t *)malloc((size_t)(chunk * orb));
    if (!buf) return fail("out of host memory", NULL);
    gp_host_register(buf, (size_t)(chunk * orb));
    for (int64_t s0 = 0; s0 < nkeep_snp; s0 += chunk) {
      const int64_t nc = nkeep_snp - s0 < chunk ? nkeep_snp - s0 : chunk;
      if (gp_encode_records(ctx, format, sidx, nout, sel + s0, sflip + s0, nc, buf, 0))
        return fail(gp_last_error(ctx), NULL);
      if (fwrite(buf, 1, (size_t)(nc * orb), f) != (size_t)(nc * orb))
        return fail("write failed: ", gout);
    }
    gp_host_unregister(buf);
    free(buf);
    fclose(f);
  }
  printf("##end of gpuconvertf run\n");
  gp_close(ctx);
  gp_free_snps(&snps);
  gp_free_inds(&inds);
  gp_par_free(&pf);
  return 0;
}
