/*
 * gpupca.h — C ABI of the GB300 (sm_103a) smartpca hot path.
 *
 * The reference smartpca (EIGENSOFT 8.0.0) has no plugin API: its hot path is a set of
 * internal C functions called from main() in src/eigensrc/smartpca.c with globals as
 * hidden parameters.  Each entry point below replaces one of them and says which
 * (file:line in the reference).  Conventions:
 *
 *   * every call returns int status: GP_OK (0) or a negative GP_ERR_* code; nothing exits
 *     the process (the reference calls fatalx/exit);  gp_last_error() has the message;
 *   * buffers passed in and out are caller-owned HOST memory with plain C types; the
 *     genotype panel, the Gram matrix and the eigenvectors live in device memory owned by
 *     the handle, which does all of its work on its own CUDA stream;
 *   * one handle is used by one host thread at a time; separate handles are independent.
 *
 * Genotype codes: per sample a 2-bit count of the FIRST allele 0/1/2, 3 = missing, packed
 * four samples per byte, sample k at byte k>>2, bits (3-(k&3))*2 (packedancestrymap,
 * src/admutils.c:718-735), or the PLINK .bed code (LSB first, 00->2, 01->missing, 10->1,
 * 11->0, src/mcio.c:3995-4009) which is recoded on upload.
 */
#ifndef GPUPCA_H
#define GPUPCA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GP_OK 0
#define GP_ERR_ARG (-1)      /* bad argument or size */
#define GP_ERR_CUDA (-2)     /* CUDA runtime / launch failure */
#define GP_ERR_NOMEM (-3)    /* device or host allocation failed */
#define GP_ERR_STATE (-4)    /* call out of order (e.g. no genotypes loaded) */
#define GP_ERR_SOLVER (-5)   /* eigensolver / factorisation failure */
#define GP_ERR_NODATA (-6)   /* zero or NaN trace: "XTX has zero trace (perhaps no data)" */
#define GP_ERR_TIMEOUT (-7)  /* bounded device wait ran out (serving loop) */
#define GP_ERR_FULL (-8)     /* serving: no slot or memory free for the request */
#define GP_ERR_NOTBUILT (-9) /* feature not compiled into this library */

#define GP_CODE_PACKED 0     /* packedancestrymap 2-bit, MSB first, 3 = missing */
#define GP_CODE_BED 1        /* PLINK .bed, LSB first, 01 = missing */

#define GP_PREC_FP64 0         /* plain FP64 Gram: the drop-in */
/* Split precisions: each normalised value v = hi + lo in a 16-bit format, tcgen05 MMAs with
 * FP32 accumulation inside a SNP chunk and FP64 accumulation across chunks. */
#define GP_PREC_SPLIT_BF16 1   /* bf16 hi+lo, 3 MMAs (hi.hi + hi.lo + lo.hi): the dropped
                                  lo.lo term biases eigenvalues low by ~2^-18 (~4e-6) */
#define GP_PREC_SPLIT_BF16X4 2 /* bf16 hi+lo, 4 MMAs (adds lo.lo): no bias, 4/3 the MMAs */
#define GP_PREC_SPLIT_FP16 3   /* fp16 hi+lo (11-bit halves), 3 MMAs: lo.lo ~2^-22 */

typedef struct gp_ctx gp_ctx;

/* Library version (major*10000 + minor*100 + patch) and the last error text of a handle
 * (or of the last failed gp_open when ctx is NULL). */
int gp_version(void);
const char *gp_last_error(const gp_ctx *ctx);

/* Open a handle on CUDA device `device` (creates its stream and solver handles). */
int gp_open(int device, gp_ctx **out);
void gp_close(gp_ctx *ctx);

/* Device memory the handle currently holds, in bytes. */
int gp_device_bytes(const gp_ctx *ctx, int64_t *bytes);

/*
 * Upload the genotype panel: nsnp records of record_bytes bytes, SNP-major, in the order
 * of the caller's SNP list (after the reference's (chrom, genpos, physpos) sort), nind
 * samples each.  Replaces reading packgenos into cupt->pbuff (inpack src/mcio.c:2769-2865)
 * and the BED re-encode (getbedgenos src/mcio.c:3893-3992).  Invalidates earlier sample and
 * SNP selections.
 */
int gp_load_genotypes(gp_ctx *ctx, const uint8_t *records, int64_t record_bytes,
                      int64_t nsnp, int32_t nind, int32_t code);

/* Shape of the resident panel (0 when none is loaded). */
int gp_genotype_shape(const gp_ctx *ctx, int64_t *nsnp, int32_t *nind);

/*
 * Set a genotype to missing in the device panel (the male-X-het rule, checkxval
 * src/mcio.c:1606-1619, applied by putgtypes(cupt, k, -1) in inpack :2856-2863).
 * pairs = npairs (snp, sample) index pairs.
 */
int gp_set_missing(gp_ctx *ctx, const int64_t *pairs, int64_t npairs);

/*
 * missingmode: replace every genotype of the resident panel by the indicator of its being
 * observed (1 for 0/1/2, 0 for missing), as setmiss does (src/qpsubs.c:462-483, called at
 * src/eigensrc/smartpca.c:901-904 after the pre-filters; the caller then runs with
 * fancynorm off).
 */
int gp_set_missingmode(gp_ctx *ctx);

/*
 * Valid-genotype counts used by the reference's pre-filters: per SNP over the samples with
 * sample_use[k] != 0 (numvalidgtx src/admutils.c:1136, numvalidgt :1118), and per sample over
 * the SNPs with snp_use[s] != 0 (numvalidgtallind :1075).  Either output may be NULL.
 */
int gp_valid_counts(gp_ctx *ctx, const uint8_t *sample_use, const uint8_t *snp_use,
                    int32_t *snp_valid, int32_t *sample_valid);

/* The rows of the analysis: ascending sample indices (loadindx src/qpsubs.c:202). */
int gp_set_samples(gp_ctx *ctx, const int32_t *xindex, int32_t nrows);

/* The columns of the analysis: SNP indices into the loaded records (loadsnpx
 * src/qpsubs.c:222). */
int gp_set_snps(gp_ctx *ctx, const int32_t *snp_index, int32_t ncols);

typedef struct {
  int32_t fancynorm;    /* usenorm / fancynorm (default 1): divide by sqrt(p(1-p)) */
  int32_t altnormstyle; /* altnormstyle (default 1): p = mean/2, else (c0+1)/(2n+2) */
  int32_t minallelecnt; /* default 1 */
  int32_t maxmissing;   /* default 9999999 */
  int32_t precision;    /* GP_PREC_FP64 or GP_PREC_SPLIT_BF16 */
} gp_xtx_opts;

/*
 * One Gram pass of the outlier loop over the current rows and columns.  Per selected SNP:
 * counts n0 = sum g, n1 = sum (2-g), nmiss over the rows (getcolxz_binary1
 * src/eigensrc/smartpca.c:3219-3301), the kill rule min(n0,n1) < minallelecnt,
 * nmiss > maxmissing, min == 0 or no data (:1131-1144), the normalised value table
 * (fvadjust_binary :2282-2313), then XTX = sum over kept SNPs of v v^T
 * (domult_increment_lookup :3426 / domult_increment_normal :3531, symit2 :480).
 * Outputs (host, may be NULL): n0, n1, nmiss, killed [ncols]; xmean = mean*fancy and
 * xfancy = fancy [ncols] (zero for a SNP with no data, as the reference);
 * XTX [nrows*nrows] full symmetric (unscaled); trace (unscaled); nused = kept SNPs.
 * The Gram stays resident in device memory for gp_eigvecs.
 */
int gp_xtx(gp_ctx *ctx, const gp_xtx_opts *opts, int32_t *n0, int32_t *n1, int32_t *nmiss,
           uint8_t *killed, double *xmean, double *xfancy, double *XTX, double *trace,
           int32_t *nused);

/*
 * Scale the resident Gram by (nrows-1)/trace (smartpca.c:1230-1236) and solve the dense
 * symmetric eigenproblem in FP64 on the device (eigvecs src/eigensrc/eigsubs.c:39-55 ->
 * dspev).  evals [nrows] all eigenvalues in descending order; evecs [nvec*nrows] the top
 * nvec eigenvectors, eigenvector j at evecs[j*nrows] with unit norm (sign is arbitrary, as
 * with LAPACK).  Either output may be NULL; the top nvec vectors stay resident for
 * gp_snp_weights.
 */
int gp_eigvecs(gp_ctx *ctx, int32_t nvec, double *evals, double *evecs);

/*
 * Outlier z-scores (ridoutlier src/eigensrc/smartsubs.c:18-91), a host function: for each
 * of the first neigs eigenvectors (evecs[i*n..]) z = (v - mean)/sd with sd over n; mode 0
 * flags |z| > thresh, mode 1 is the leave-one-out variant, mode >= 2 flags nothing.
 * badlist receives the flagged rows ascending; vecno/score the first eigenvector that
 * flagged each row (may be NULL, size n).  Returns the number flagged (>= 0) or an error.
 */
int gp_ridoutlier(const double *evecs, int32_t n, int32_t neigs, double thresh, int32_t mode,
                  int32_t *badlist, int32_t *vecno, double *score);

/*
 * SNP weights and sample scores after the last pass (smartpca.c:1485-1525): with
 * fvecs = 10*evecs (setfvecs src/qpsubs.c:489), ffvecs[j*ncols+s] = sum_k fvecs_j[k] x_s[k]
 * over the rows (killed SNPs give 0), fxvecs[j*nrows+i] = xrow_i . ffvecs_j (fixxrow
 * src/qpsubs.c:338) and fxscal[j] = 1/sqrt(sum_i fxvecs^2).  Uses the resident top
 * eigenvectors of gp_eigvecs.  Outputs may be NULL except fxscal.
 */
int gp_snp_weights(gp_ctx *ctx, int32_t numeigs, double *ffvecs, double *fxvecs,
                   double *fxscal);

/*
 * lsqproject (lsqproj src/eigensrc/smartpca.c:4606-4757 -> regressit src/regsubs.c:8 ->
 * solvit/choldc/cholsl src/nicksrc/linsubs.c:296-380): for each listed sample, over the
 * kept columns where it has a genotype, solve the masked normal equations
 * (E^T E) a = E^T r with E_sj = fxscal_j ffvecs_js and r_s = g fancy_s - xmean_s by
 * Cholesky; b_j = fxscal_j (xrow . ffvecs_j) is the orthogonal projection.
 * samples [nproj] indices into the loaded samples; acoeffs/bcoeffs [numeigs*nproj]
 * (coefficient j of sample q at [j*nproj+q]); nobs [nproj] observed kept SNPs;
 * status [nproj]: 0 ok, 1 = nobs <= numeigs (sample dropped, "insufficient data"),
 * 2 = not positive definite (acoeffs left untouched, as the reference keeps the previous
 * regans).  Requires gp_snp_weights first.  Outputs other than acoeffs may be NULL.
 */
int gp_lsqproj(gp_ctx *ctx, int32_t numeigs, const int32_t *samples, int32_t nproj,
               double *acoeffs, double *bcoeffs, int32_t *nobs, int32_t *status);

/*
 * usepopsformissing (smartpca's parfile option; FP64 precision only).
 *
 * gp_set_row_pops: the population index of each current row (row_pop [nrows]: the xtypes
 * value, smartpca.c:1095-1099; < 0 = none) and npop > every index.  The next gp_xtx then
 * fills a missing genotype of a row with its population's mean genotype over the rows
 * observed in that column (getcolxz smartpca.c:3141-3184); the column's mean and fancy scale
 * run over the observed and filled values in row order (fvadjust :2236-2279), and the kill
 * rule's missing count is the count still missing after the fill.  The SNP weights keep the
 * observed-only table (getcolxf :3564-3592); xmean/xfancy of gp_xtx are the filled ones.
 * gp_set_samples turns the option off (call this after it); NULL or npop <= 0 turns it off.
 *
 * gp_lsqproj_pops: gp_lsqproj with lsqproj's fill (smartpca.c:4631-4746): sample_pop [nproj]
 * is the population index the reference reads for each sample (xtypes at the sample's .ind
 * index; < 0 = none).  Samples with at most numeigs observed genotypes are dropped
 * (status 1) before the population sums; the others with a population add their observed
 * genotypes to it, and a missing genotype of a sample whose population has observed ones in
 * that column is filled with their mean and counts as observed (nobs includes it).
 */
int gp_set_row_pops(gp_ctx *ctx, const int32_t *row_pop, int32_t npop);
int gp_lsqproj_pops(gp_ctx *ctx, int32_t numeigs, const int32_t *samples,
                    const int32_t *sample_pop, int32_t npop, int32_t nproj, double *acoeffs,
                    double *bcoeffs, int32_t *nobs, int32_t *status);

/*
 * fastmode randomized block-Krylov PCA (kjg_fpca src/ksrc/kjg_fpca.c:24-102 with the data
 * table of setgval src/gval.c:31-87) over the current rows and columns: X (ncols x nrows)
 * holds ((g - mean) fancy)/sqrt(2), missing 0 (opts: fancynorm, altnormstyle and precision
 * are used; no allele-count kill rule applies, as in the reference); Omega (nrows x L)
 * Gaussian from `seed` (or the caller's omega, row-major, when not NULL); I power steps
 * G <- X^T X G / M; Q = [X G_0 .. X G_I] (needs (I+1) L <= 1024); Q <- orthonormal basis;
 * B = X^T Q; SVD(B).  evals [K] = S^2/M, evecs [K*nrows] (vector j at [j*nrows], unit norm,
 * arbitrary sign).  The products with X are the exact tensor-core products for split
 * precisions (FP64 SIMT for GP_PREC_FP64); orthogonalisation and Rayleigh-Ritz are FP64.
 */
int gp_fastpca(gp_ctx *ctx, int32_t K, int32_t L, int32_t I, uint64_t seed,
               const double *omega, const gp_xtx_opts *opts, double *evals, double *evecs);


/*
 * Relatedness (smartrel, src/eigensrc/smartrel.c:578-615).  gp_keep_gram(ctx, 1) makes
 * gp_eigvecs keep a device copy of the scaled Gram; gp_relate then removes the top numeigs
 * components, R = XTX - sum_i lambda_i v_i v_i^T (subouter, in order), and returns the row
 * pairs a < b (indices into the PCA rows) with y = R_ab / sqrt(R_aa R_bb) + 1/(nrows-1) >=
 * relthresh, in no particular order (the caller sorts by y, as the reference prints them).
 * *npairs is the number found; at most max_pairs are copied.
 */
int gp_keep_gram(gp_ctx *ctx, int32_t keep);
int gp_relate(gp_ctx *ctx, int32_t numeigs, double relthresh, int64_t max_pairs,
              int32_t *pair_a, int32_t *pair_b, double *score, int64_t *npairs);

/*
 * Genotype record writers of convertf (outputformat:) from the resident panel.
 * gp_record_bytes: bytes of one output record for nsamples samples (-1 for a bad format):
 *   GP_OUT_PACKEDANCESTRYMAP  max(ceil(n/4), 48)  outpack        src/mcio.c:2343-2457
 *   GP_OUT_PACKEDPED          ceil(n/4)           outpackped     src/mcio.c:3619-3741
 *   GP_OUT_EIGENSTRAT         n + 1 ('0'-'2', '9' missing, '\n') outeigenstrat src/mcio.c:3262
 * gp_encode_records writes nsnps records (SNP snp_index[i] of the panel, samples
 * sample_index[0..nsamples) in that order, or samples 0..nsamples-1 when sample_index is
 * NULL; flip[i] != 0 replaces each observed g by 2 - g as flip1 does,
 * src/convertf.c:1017-1026) to out (host memory, or device memory when out_on_device), one
 * record after another.  The file headers (the "GENO" record, the bed magic) are the
 * caller's.
 */
#define GP_OUT_PACKEDANCESTRYMAP 0
#define GP_OUT_PACKEDPED 1
#define GP_OUT_EIGENSTRAT 2
int64_t gp_record_bytes(int32_t format, int32_t nsamples);
int gp_encode_records(gp_ctx *ctx, int32_t format, const int32_t *sample_index,
                      int32_t nsamples, const int64_t *snp_index, const uint8_t *flip,
                      int64_t nsnps, uint8_t *out, int32_t out_on_device);

/*
 * Fst between populations over the columns of the last gp_xtx pass that were not killed and
 * the current rows (dofstxx src/eigensrc/smartpca.c:2830-2878, dofstnumx src/qpsubs.c:2488-2720,
 * fstcolyy :1205-1345): xtypes[r] is the population (0..numeg-1; other values: none) of row r,
 * snp_block[s] the jackknife block of panel SNP s (-1: none; gp_set_blocks), nblocks the
 * number of blocks (numblocks :1631).  Per population pair a < b: fstnum = SNPs with an
 * estimate, fstmean = sum N / (sum D + 1e-10), fstans and fstsd the weighted block-jackknife
 * estimate and standard error (wjackest :2793-2858; fstmean and 0 with one block); all four
 * [numeg*numeg] symmetric with a zero diagonal (fstmean: upper triangle).  Any output may be NULL.
 * Populations are counted on the device; the estimator and jackknife run on the host in the
 * reference's operation order.
 */
int gp_fst(gp_ctx *ctx, const int32_t *xtypes, int32_t numeg, const int32_t *snp_block,
           int32_t nblocks, double *fstmean, double *fstans, double *fstsd, int32_t *fstnum);

/* setblocks (src/qpsubs.c:1578-1627), a host function: block tags for n SNPs in sorted order
 * (a new block at a chromosome change or blocklen morgans after the block's first SNP; SNPs
 * with ignore[i] set get -1; tag may be NULL).  Returns the number of blocks. */
int32_t gp_set_blocks(const int32_t *chrom, const double *gpos, const uint8_t *ignore, int64_t n,
                      double blocklen, int32_t *tag);

/* Free every device buffer of the handle (panel, Gram, vectors, scratch); the handle, its
 * stream and solver stay usable and the next gp_load_genotypes starts afresh.  No
 * counterpart in the reference (a process ends instead). */
int gp_release(gp_ctx *ctx);

/* ---- measurement helpers (no counterpart in the reference) ---------------------------- */

/* Device stopwatch on the handle's stream (CUDA events); stop synchronises the stream. */
int gp_timer_start(gp_ctx *ctx);
int gp_timer_stop(gp_ctx *ctx, double *ms);

/* Device time of the Gram kernel launches of the last gp_xtx call (CUDA events around them
 * on the handle's stream), the number of Gram-kernel launches, and the algorithmic flop
 * count nrows*(nrows+1)*kept_snps of that call. */
int gp_last_gram_time(const gp_ctx *ctx, double *ms, int32_t *launches, double *flops);

/* Device time of the tridiagonalisation kernel (k_tridiag) of the last eigensolve (CUDA events
 * around its launch on the handle's stream) and the matrix order; 0 ms when that solve used
 * cuSOLVER's sytrd instead. */
int gp_last_tridiag_time(const gp_ctx *ctx, double *ms, int32_t *n);

/* Device time of the per-SNP counts kernel (k_snp_stats) of the last pass (CUDA events around
 * its launch on the handle's stream; waits for it) and its algorithmic bytes: one read of
 * each selected record and of the row mask, 61 bytes of counts and tables written per SNP. */
int gp_last_counts_time(const gp_ctx *ctx, double *ms, int64_t *bytes);

/* Device time of the k_encode launch of the last gp_encode_records call that wrote to
 * device memory (CUDA events around it on the handle's stream). */
int gp_last_encode_time(const gp_ctx *ctx, double *ms);

/* Host->device and device->host bytes the handle has copied (optionally reset to 0). */
int gp_transfer_bytes(gp_ctx *ctx, int64_t *h2d, int64_t *d2h, int32_t reset);

/* Number of this library's own kernels the handle has launched (optionally reset). */
int gp_launch_count(gp_ctx *ctx, int64_t *launches, int32_t reset);

/* Page-lock a host buffer for fast uploads (cudaHostRegister) and release it. */
int gp_host_register(void *ptr, size_t bytes);
int gp_host_unregister(void *ptr);

/* ---- no-allocation entry point (no counterpart in the reference) ----------------------- */

/*
 * FP64 Gram XTX = sum over SNPs s of v_s v_s^T for a small panel, computed without any
 * device allocation, for callers that cannot allocate: e.g. a process whose memory manager
 * has reserved the whole device for its own pool, or a latency-critical loop that must not
 * call cudaMalloc/cudaFree (they can synchronise the device).  All buffers are the caller's
 * DEVICE memory: d_records = nsnp packed records of record_bytes bytes (2-bit
 * packedancestrymap code, every sample and SNP used), d_vtab = [4*nsnp] value of codes
 * 0,1,2,3 per SNP (as gp_xtx builds them; 3 = missing, normally 0), d_xtx = [nind*nind]
 * output, full symmetric.  Work is queued on `stream` (a cudaStream_t; NULL = default).
 * Limit: nind <= 1024 (larger panels return GP_ERR_ARG; use gp_xtx).  Scratch for the
 * split-K partial sums is a fixed 16 MiB array inside the library that every GPU loading it
 * holds until exit; the first call on a device looks its address up (make it before any
 * stream capture) and, as CUDA loads modules lazily by default, is also when the array is
 * allocated on that device: make the first call before a pool reserves the whole device.
 * Each call overwrites the scratch entries it reads; calls that overlap on the GPU race on
 * that array.  The cached address is not refreshed after cudaDeviceReset (do not call the
 * entry point again on a device that was reset).  The host side may be called from several
 * threads; gp_noalloc_last_error gives the text of the calling thread's last failure.
 */
int gp_gram_fp64_noalloc(const uint8_t *d_records, int64_t record_bytes, int32_t nind,
                         int32_t nsnp, const double *d_vtab, double *d_xtx, void *stream);
const char *gp_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* GPUPCA_H */
