/* Internal state of a gpupca handle and helpers shared by the .cu files. */
#ifndef GP_INTERNAL_H
#define GP_INTERNAL_H

#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <vector>

#include "../../include/gpupca.h"

#define GP_ERRLEN 512

struct gp_ctx {
  int device;
  int num_sms;
  cudaStream_t stream;
  cusolverDnHandle_t solver;
  cublasHandle_t blas;  /* created on first use (fastmode) */
  char err[GP_ERRLEN];

  /* genotype panel: nsnp_all records of rlen_dev bytes (packed 2-bit, MSB first) */
  uint8_t *d_geno;
  size_t geno_cap;   /* bytes allocated at d_geno */
  int64_t nsnp_all;
  int32_t nind_all;
  int64_t rlen_dev;  /* padded to a multiple of 16 bytes; pad bytes are 0xFF (missing) */

  /* analysis rows/columns */
  int32_t *d_rows;       /* [nrows] ascending sample indices */
  uint32_t *d_rowmask;   /* [rlen_dev/4] 2-bit selection mask (0b11 per selected sample) */
  int32_t nrows;
  int32_t *d_cols;       /* [ncols] SNP indices into the records */
  int32_t ncols;

  /* per-column state of the last gp_xtx */
  int32_t *d_cnt;        /* [3*ncols]: n0, n1, nmiss */
  uint8_t *d_killed;     /* [ncols] */
  double *d_vtab;        /* [4*ncols]: value of code 0,1,2,3(missing)=0 */
  double *d_xmean;       /* [ncols] */
  double *d_xfancy;      /* [ncols] */
  int32_t *d_kept;       /* [ncols] compacted list of kept columns (positions in cols) */
  int32_t nkept;
  /* usepopsformissing (gp_set_row_pops): the rows' population indices and, after gp_xtx,
   * the Gram's table of the filled column and the populations' fill values */
  int32_t *d_rowpop;     /* [nrows] (< 0: no population) */
  int32_t npop;          /* 0: off (gp_set_samples turns it off) */
  double *d_gtab;        /* [4*ncols] */
  double *d_gfill;       /* [ncols*npop] */
  int xtx_valid;
  double trace;        /* unscaled trace of the last Gram */

  /* Gram and eigen state */
  double *d_xtx;         /* [nrows*nrows] */
  int64_t xtx_cap;
  double *d_evals;       /* [nrows] */
  double *d_evecs;       /* [nvec*nrows] top vectors, descending */
  double *d_tri;         /* the tiled tridiagonalisation's lower-triangle tiles and parts */
  unsigned char *d_tt;   /* its assignment tables, for order tt_n on a grid of tt_G blocks */
  int tt_n, tt_G, tt_maxr, tt_maxc, tt_maxi;
  int keep_gram;         /* gp_keep_gram: copy the scaled Gram before the eigensolve */
  double *d_xtx_keep;    /* [nrows*nrows] that copy (the relatedness scan reads it) */
  int64_t keep_cap;
  int keep_valid;
  int32_t nvec;
  int eig_valid;

  /* weights */
  double *d_ffvecs;      /* [nvec*ncols] */
  double *d_fxscal;      /* [nvec] */
  int weights_valid;
  int32_t nweights;

  /* timing */
  cudaEvent_t ev_t0, ev_t1, ev_g0, ev_g1;
  double gram_ms;
  int32_t gram_launches;
  int gram_cluster_cap;  /* largest split-Gram cluster size to try (0: 4); set to 1 after a
                            cluster launch was not honoured */
  double gram_flops;
  double encode_ms;      /* k_encode time of the last device-output gp_encode_records */
  cudaEvent_t ev_tr0, ev_tr1;
  cudaEvent_t ev_c0, ev_c1; /* around the last k_snp_stats launch */
  int64_t counts_bytes;     /* its algorithmic bytes (0: none yet) */
  double tridiag_ms;     /* k_tridiag time of the last eigensolve (0: cuSOLVER sytrd ran) */
  int32_t tridiag_n;     /* its order */

  /* host<->device bytes copied by the handle (gp_transfer_bytes) */
  int64_t h2d_bytes, d2h_bytes;
  int64_t launches;   /* kernels of this library launched by the handle */

  /* scratch arena (grows on demand, freed at close) */
  void *d_scratch;
  size_t scratch_cap;
  void *d_scratch2;
  size_t scratch2_cap;
  void *d_scratch3;    /* small panels built between the products of gp_geno_tc */
  size_t scratch3_cap;
  void *d_scratch4;    /* genotype code operands of gp_geno_tc */
  size_t scratch4_cap;
  int codes4_rows;     /* d_scratch4 holds the sample-major codes of the current rows over the
                          kept columns of the last gp_xtx, for reuse by the next product */
  int32_t *h_rows;     /* [nrows] host copy of d_rows */
  void *d_scratch5;    /* exact integer partial sums of gp_geno_tc */
  size_t scratch5_cap;
  int *d_err;          /* error word written by the tensor-core kernels' bounded waits */
  int precision;       /* precision of the last gp_xtx: split precisions use the tensor-core
                          exact products for weights and lsqproject */
  /* capacities of the buffers gp_realloc manages (kept while large enough) */
  struct {
    void **p;
    size_t bytes;
  } caps[32];
  int ncaps;
};

int gp_fail(gp_ctx *ctx, int code, const char *fmt, ...);
/* cudaMemcpyAsync that also counts host<->device bytes on the handle */
cudaError_t gp_memcpy(gp_ctx *ctx, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind,
                      cudaStream_t stream);
int gp_cuda_fail(gp_ctx *ctx, cudaError_t e, const char *what);
int gp_scratch(gp_ctx *ctx, size_t bytes, void **out);
int gp_scratch2(gp_ctx *ctx, size_t bytes, void **out);
int gp_scratch_aux(gp_ctx *ctx, size_t bytes, void **out);
int gp_scratch4(gp_ctx *ctx, size_t bytes, void **out);
int gp_scratch5(gp_ctx *ctx, size_t bytes, void **out);
int gp_realloc(gp_ctx *ctx, void **ptr, size_t bytes);
/* allow a kernel the device's largest dynamic shared memory (the opt-in maximum less its static
 * shared memory).  The limit is a process-wide attribute of the function: setting it to one
 * fixed value instead of each call's own size keeps concurrent handles (serving workers) from
 * lowering it between another call's check and launch.  Each launch still requests, and
 * occupies, only its own size. */
cudaError_t gp_allow_smem(gp_ctx *ctx, const void *func);

#define GP_CUDA(ctx, call)                                   \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return gp_cuda_fail(ctx, _e, #call); \
  } while (0)

#define GP_LAUNCH_CHECK(ctx, what)                          \
  do {                                                       \
    (ctx)->launches++;                                       \
    cudaError_t _e = cudaGetLastError();                     \
    if (_e != cudaSuccess) return gp_cuda_fail(ctx, _e, what); \
  } while (0)

/* kernels, by file */
int gp_launch_valid_counts(gp_ctx *ctx, const uint8_t *d_sample_use, const uint8_t *d_snp_use,
                           int32_t *d_snp_valid, int32_t *d_sample_valid);
int gp_launch_snp_stats(gp_ctx *ctx, const gp_xtx_opts *o);
/* usepopsformissing (gp_popfill.cu): the filled Gram tables of a pass, and lsqproj's fill
 * tables (work: gp_lsq_fill_work_bytes; raw = observed kept genotypes per sample) */
int gp_popfill_pass(gp_ctx *ctx, const gp_xtx_opts *o);
size_t gp_lsq_fill_work_bytes(int32_t nproj, int32_t nk, int32_t npop);
int gp_lsq_fill_tables(gp_ctx *ctx, const int32_t *d_samp, const int32_t *d_spop, int32_t nproj,
                       int32_t npop, int32_t K, const int32_t *d_snprec, const double *d_ot,
                       int32_t nk, void *work, double **d_raw, double **d_of, double **d_rf);
int gp_gram_fp64(gp_ctx *ctx);
int gp_gram_split(gp_ctx *ctx, int precision);
int gp_launch_symmetrize_trace(gp_ctx *ctx, double *d_trace);
int gp_eig_tridiag(gp_ctx *ctx, int32_t n, int32_t nvec, double *d_evals_desc, double *d_vecs);
int gp_eig_sym(gp_ctx *ctx, double *A, int32_t n, int32_t nvec, double *d_evals_desc,
               double *d_vecs);
/* per-sample masked normal equations solve of lsqproj (gp_api.cu); co rows hold the K(K+1)/2
 * pair sums then the observed count, rr rows the K right-hand sides; acoef/bcoef are [K][nproj];
 * d_nproj (device, may be NULL) replaces nproj at run time */
__global__ void k_lsq_solve(const double *co, int32_t ldco, const double *rr, int32_t K,
                            int32_t nproj, double *acoef, double *bcoef, int32_t *nobs,
                            int32_t *status, double *work, const int32_t *d_nproj);
int gp_launch_materialize_f64(gp_ctx *ctx, int32_t k0, int32_t kc, int32_t pitch, double *d_x,
                              double scale);

#endif
