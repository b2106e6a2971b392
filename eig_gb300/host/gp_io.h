/* File formats of the smartpca drop-in: parfile, SNP/sample lists, genotype files. */
#ifndef GP_IO_H
#define GP_IO_H

#include <stdint.h>

#define GP_IDLEN 64

typedef struct {
  int n;
  char **key;   /* with the trailing ':' */
  char **val;
} gp_parfile;

int gp_par_read(const char *path, gp_parfile *pf);
void gp_par_free(gp_parfile *pf);
/* 1 when found; YES/NO map to 1/0 for ints */
int gp_par_int(const gp_parfile *pf, const char *key, int32_t *out);
int gp_par_dbl(const gp_parfile *pf, const char *key, double *out);
int gp_par_str(const gp_parfile *pf, const char *key, const char **out);

typedef struct {
  int64_t n;
  char (*id)[GP_IDLEN];
  int32_t *chrom;
  double *gpos;
  double *ppos;
  char (*alleles)[2]; /* first (reference) and second allele; 0 when the file has none */
  int64_t *order;   /* sorted position -> input row */
} gp_snplist;

typedef struct {
  int32_t n;
  char (*id)[GP_IDLEN];
  char *gender;
  char (*pop)[GP_IDLEN];
  uint8_t *ignore;
} gp_indlist;

int gp_read_snps(const char *path, int numchrom, gp_snplist *s, char *err, int errlen);
int gp_read_inds(const char *path, int familynames, gp_indlist *ind, char *err, int errlen);
void gp_free_snps(gp_snplist *s);
void gp_free_inds(gp_indlist *ind);

/*
 * Genotypes for all SNPs in sorted order as packed records: out_records (nsnp x rec_bytes)
 * and the code (GP_CODE_PACKED, or GP_CODE_BED which the device recodes).  Reads
 * packedancestrymap (GENO header, hash check optional), PLINK .bed and EIGENSTRAT text.
 */
int gp_read_genotypes(const char *path, const gp_snplist *s, const gp_indlist *ind,
                      int hashcheck, uint8_t **out_records, int64_t *rec_bytes, int32_t *code,
                      char *err, int errlen);

/*
 * GRM dump of the last pass (dumpgrm/dumpgrmbin/dumpgrmid src/eigensrc/smartpca.c:3687-3808)
 * from the unscaled XTX (n x n, row-major): the Gram is first scaled by (n-1)/trace as the
 * PCA does (:1230-1236), then written as GCTA text "i j numsnps value" (lower triangle,
 * value = XTX * n / sum(diag)) or, with binary = 1, as name.bin (float, XTX / (trace/n)) and
 * name.N.bin (int32 numsnps, n(n+1)/2 times); name.id gets "NA\tID" per row.
 */
int gp_write_grm(const char *name, int binary, const double *xtx, int32_t n, int32_t numsnps,
                 char (*ids)[GP_IDLEN], const int32_t *xindex, char *err, int errlen);

#endif
