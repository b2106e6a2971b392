/*
 * C ABI of the smartpca hot path: handle management and the pass orchestration
 * (gp_xtx, gp_eigvecs, gp_snp_weights, gp_lsqproj) plus the host-side outlier rule.
 * The numerical work runs in the kernels of the other .cu files on the handle's stream.
 */
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <algorithm>
#include <vector>

#include "gp_geno_gemm.h"
#include "gp_geno_tc.h"
#include "gp_internal.h"

#define GP_VERSION 10000

static char g_open_err[GP_ERRLEN];

extern "C" int gp_version(void) { return GP_VERSION; }

extern "C" const char *gp_last_error(const gp_ctx *ctx) { return ctx ? ctx->err : g_open_err; }

int gp_fail(gp_ctx *ctx, int code, const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(ctx ? ctx->err : g_open_err, GP_ERRLEN, fmt, ap);
  va_end(ap);
  return code;
}

extern "C" int gp_fail_msg(gp_ctx *ctx, int code, const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(ctx ? ctx->err : g_open_err, GP_ERRLEN, fmt, ap);
  va_end(ap);
  return code;
}

cudaError_t gp_memcpy(gp_ctx *ctx, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind,
                      cudaStream_t stream)
{
  if (kind == cudaMemcpyHostToDevice) ctx->h2d_bytes += (int64_t)bytes;
  if (kind == cudaMemcpyDeviceToHost) ctx->d2h_bytes += (int64_t)bytes;
  return cudaMemcpyAsync(dst, src, bytes, kind, stream);
}

int gp_cuda_fail(gp_ctx *ctx, cudaError_t e, const char *what)
{
  return gp_fail(ctx, e == cudaErrorMemoryAllocation ? GP_ERR_NOMEM : GP_ERR_CUDA,
                 "%s: %s", what, cudaGetErrorString(e));
}

static int grow(gp_ctx *ctx, void **buf, size_t *cap, size_t bytes)
{
  if (bytes <= *cap && *buf) return GP_OK;
  if (*buf) {
    cudaFree(*buf);
    *buf = NULL;
    *cap = 0;
  }
  size_t want = bytes < 256 ? 256 : bytes;
  cudaError_t e = cudaMalloc(buf, want);
  if (e != cudaSuccess) {
    *buf = NULL;
    return gp_fail(ctx, GP_ERR_NOMEM, "device allocation of %zu bytes failed: %s", want,
                   cudaGetErrorString(e));
  }
  *cap = want;
  return GP_OK;
}

int gp_scratch(gp_ctx *ctx, size_t bytes, void **out)
{
  int rc = grow(ctx, &ctx->d_scratch, &ctx->scratch_cap, bytes);
  *out = ctx->d_scratch;
  return rc;
}

int gp_scratch_aux(gp_ctx *ctx, size_t bytes, void **out)
{
  int rc = grow(ctx, &ctx->d_scratch3, &ctx->scratch3_cap, bytes);
  *out = ctx->d_scratch3;
  return rc;
}

int gp_scratch4(gp_ctx *ctx, size_t bytes, void **out)
{
  ctx->codes4_rows = 0; /* the caller overwrites the codes */
  int rc = grow(ctx, &ctx->d_scratch4, &ctx->scratch4_cap, bytes);
  *out = ctx->d_scratch4;
  return rc;
}

int gp_scratch5(gp_ctx *ctx, size_t bytes, void **out)
{
  int rc = grow(ctx, &ctx->d_scratch5, &ctx->scratch5_cap, bytes);
  *out = ctx->d_scratch5;
  return rc;
}

int gp_scratch2(gp_ctx *ctx, size_t bytes, void **out)
{
  int rc = grow(ctx, &ctx->d_scratch2, &ctx->scratch2_cap, bytes);
  *out = ctx->d_scratch2;
  return rc;
}

/* a handle buffer of at least `bytes` (contents not kept): the allocation stays while it is
 * large enough, so that the per-pass buffers of a run (sample and SNP lists, tables, vectors)
 * cost no cudaFree / cudaMalloc, nor their device synchronisation, after the first pass */
int gp_realloc(gp_ctx *ctx, void **ptr, size_t bytes)
{
  if (bytes < 256) bytes = 256;
  int slot = -1;
  for (int i = 0; i < ctx->ncaps; ++i)
    if (ctx->caps[i].p == ptr) slot = i;
  if (slot >= 0 && *ptr && ctx->caps[slot].bytes >= bytes) return GP_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = NULL;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = NULL;
    return gp_fail(ctx, GP_ERR_NOMEM, "device allocation of %zu bytes failed: %s", bytes,
                   cudaGetErrorString(e));
  }
  if (slot < 0 && ctx->ncaps < (int)(sizeof(ctx->caps) / sizeof(ctx->caps[0]))) {
    slot = ctx->ncaps++;
    ctx->caps[slot].p = ptr;
  }
  if (slot >= 0) ctx->caps[slot].bytes = bytes;
  return GP_OK;
}

cudaError_t gp_allow_smem(gp_ctx *ctx, const void *func)
{
  int optin = 0;
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                         ctx->device);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, func);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)fa.sharedSizeBytes);
}

extern "C" int gp_open(int device, gp_ctx **out)
{
  if (!out) return gp_fail(NULL, GP_ERR_ARG, "gp_open: out is NULL");
  *out = NULL;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return gp_fail(NULL, GP_ERR_CUDA, "gp_open: no CUDA device (%s)", cudaGetErrorString(e));
  if (device < 0 || device >= ndev)
    return gp_fail(NULL, GP_ERR_ARG, "gp_open: device %d out of range", device);
  gp_ctx *ctx = (gp_ctx *)calloc(1, sizeof(gp_ctx));
  if (!ctx) return gp_fail(NULL, GP_ERR_NOMEM, "gp_open: host allocation failed");
  ctx->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    gp_fail(NULL, GP_ERR_CUDA, "gp_open: %s", cudaGetErrorString(e));
    free(ctx);
    return GP_ERR_CUDA;
  }
  if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_err, 256);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_t0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_t1);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_g0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_tr0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_tr1);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_c0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_c1);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_g1);
  if (e != cudaSuccess) {
    gp_fail(NULL, GP_ERR_CUDA, "gp_open: %s", cudaGetErrorString(e));
    free(ctx);
    return GP_ERR_CUDA;
  }
  if (cusolverDnCreate(&ctx->solver) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnSetStream(ctx->solver, ctx->stream) != CUSOLVER_STATUS_SUCCESS) {
    cudaStreamDestroy(ctx->stream);
    free(ctx);
    return gp_fail(NULL, GP_ERR_SOLVER, "gp_open: cusolverDnCreate failed");
  }
  *out = ctx;
  return GP_OK;
}

extern "C" void gp_close(gp_ctx *ctx)
{
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  void *bufs[] = {ctx->d_geno,   ctx->d_rows,    ctx->d_rowmask, ctx->d_cols,    ctx->d_cnt,
                  ctx->d_killed, ctx->d_vtab,    ctx->d_xmean,   ctx->d_xfancy,  ctx->d_kept,
                  ctx->d_xtx,    ctx->d_evals,   ctx->d_evecs,   ctx->d_ffvecs,  ctx->d_fxscal,
                  ctx->d_scratch, ctx->d_scratch2, ctx->d_scratch3, ctx->d_scratch4, ctx->d_scratch5,
                  ctx->d_err,   ctx->d_xtx_keep, ctx->d_rowpop, ctx->d_gtab, ctx->d_gfill,
                  ctx->d_tri,   ctx->d_tt};
  for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); ++i)
    if (bufs[i]) cudaFree(bufs[i]);
  if (ctx->solver) cusolverDnDestroy(ctx->solver);
  if (ctx->blas) cublasDestroy(ctx->blas);
  if (ctx->ev_t0) cudaEventDestroy(ctx->ev_t0);
  if (ctx->ev_t1) cudaEventDestroy(ctx->ev_t1);
  if (ctx->ev_g0) cudaEventDestroy(ctx->ev_g0);
  if (ctx->ev_tr0) cudaEventDestroy(ctx->ev_tr0);
  if (ctx->ev_tr1) cudaEventDestroy(ctx->ev_tr1);
  if (ctx->ev_c0) cudaEventDestroy(ctx->ev_c0);
  if (ctx->ev_c1) cudaEventDestroy(ctx->ev_c1);
  if (ctx->ev_g1) cudaEventDestroy(ctx->ev_g1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  free(ctx->h_rows);
  free(ctx);
}

extern "C" int gp_release(gp_ctx *ctx)
{
  if (!ctx) return GP_ERR_ARG;
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  void **bufs[] = {(void **)&ctx->d_geno,    (void **)&ctx->d_rows,     (void **)&ctx->d_rowmask,
                   (void **)&ctx->d_cols,    (void **)&ctx->d_cnt,      (void **)&ctx->d_killed,
                   (void **)&ctx->d_vtab,    (void **)&ctx->d_xmean,    (void **)&ctx->d_xfancy,
                   (void **)&ctx->d_kept,    (void **)&ctx->d_xtx,      (void **)&ctx->d_evals,
                   (void **)&ctx->d_evecs,   (void **)&ctx->d_ffvecs,   (void **)&ctx->d_fxscal,
                   (void **)&ctx->d_scratch, (void **)&ctx->d_scratch2, (void **)&ctx->d_scratch3,
                   (void **)&ctx->d_scratch4, (void **)&ctx->d_scratch5, (void **)&ctx->d_xtx_keep,
                   (void **)&ctx->d_rowpop,  (void **)&ctx->d_gtab,     (void **)&ctx->d_gfill,
                   (void **)&ctx->d_tri,     (void **)&ctx->d_tt};
  for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); ++i) {
    if (*bufs[i]) cudaFree(*bufs[i]);
    *bufs[i] = NULL;
  }
  ctx->scratch_cap = ctx->scratch2_cap = ctx->scratch3_cap = ctx->scratch4_cap =
      ctx->scratch5_cap = 0;
  ctx->xtx_cap = 0;
  ctx->tt_n = 0;
  ctx->geno_cap = 0;
  ctx->codes4_rows = 0;
  ctx->keep_cap = 0;
  ctx->keep_valid = 0;
  ctx->nsnp_all = 0;
  ctx->nind_all = 0;
  ctx->rlen_dev = 0;
  ctx->nrows = ctx->ncols = ctx->nkept = ctx->nvec = ctx->nweights = 0;
  ctx->npop = 0;
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  return GP_OK;
}

extern "C" int gp_device_bytes(const gp_ctx *ctx, int64_t *bytes)
{
  if (!ctx || !bytes) return GP_ERR_ARG;
  int64_t b = (int64_t)ctx->rlen_dev * ctx->nsnp_all + (int64_t)ctx->scratch_cap +
              (int64_t)ctx->scratch2_cap + (int64_t)ctx->scratch3_cap +
              (int64_t)ctx->scratch4_cap + (int64_t)ctx->scratch5_cap +
              (int64_t)sizeof(double) * ctx->xtx_cap;
  *bytes = b;
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */

__global__ void k_scale(double *x, int64_t n, double s)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = x[i] * s;
}

extern "C" int gp_xtx(gp_ctx *ctx, const gp_xtx_opts *opts, int32_t *n0, int32_t *n1,
                      int32_t *nmiss, uint8_t *killed, double *xmean, double *xfancy,
                      double *XTX, double *trace, int32_t *nused)
{
  if (!ctx || !opts) return GP_ERR_ARG;
  if (!ctx->d_geno || ctx->nrows < 1 || ctx->ncols < 1)
    return gp_fail(ctx, GP_ERR_STATE, "gp_xtx: genotypes, samples and SNPs must be set first");
  if (opts->precision < GP_PREC_FP64 || opts->precision > GP_PREC_SPLIT_FP16)
    return gp_fail(ctx, GP_ERR_ARG, "gp_xtx: unknown precision %d", opts->precision);
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  const int32_t n = ctx->nrows, nc = ctx->ncols;
  int64_t need = (int64_t)n * n;
  if (need > ctx->xtx_cap) {
    int rc = gp_realloc(ctx, (void **)&ctx->d_xtx, sizeof(double) * (size_t)need);
    if (rc) {
      ctx->xtx_cap = 0;
      return rc;
    }
    ctx->xtx_cap = need;
  }
  ctx->xtx_valid = ctx->eig_valid = ctx->weights_valid = 0;
  ctx->precision = opts->precision;
  int rc;
  if (ctx->npop > 0) {
    /* usepopsformissing: the observed counts first (the missing-count rule waits for the
     * fill), then the filled tables, counts and kill flags */
    if (opts->precision != GP_PREC_FP64)
      return gp_fail(ctx, GP_ERR_ARG, "gp_xtx: usepopsformissing runs in FP64 precision only");
    gp_xtx_opts o1 = *opts;
    o1.maxmissing = 0x7FFFFFFF;
    rc = gp_launch_snp_stats(ctx, &o1);
    if (!rc) rc = gp_popfill_pass(ctx, opts);
  } else {
    rc = gp_launch_snp_stats(ctx, opts);
  }
  if (rc) return rc;

  /* kept-column list (ascending) built from the kill flags */
  std::vector<uint8_t> hk((size_t)nc);
  GP_CUDA(ctx, gp_memcpy(ctx, hk.data(), ctx->d_killed, (size_t)nc, cudaMemcpyDeviceToHost,
                               ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int32_t> kept;
  kept.reserve((size_t)nc);
  for (int32_t c = 0; c < nc; ++c)
    if (!hk[(size_t)c]) kept.push_back(c);
  ctx->nkept = (int32_t)kept.size();
  ctx->codes4_rows = 0;
  if (ctx->nkept)
    GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_kept, kept.data(), sizeof(int32_t) * kept.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));

  GP_CUDA(ctx, cudaEventRecord(ctx->ev_g0, ctx->stream));
  ctx->gram_launches = 0;
  if (opts->precision == GP_PREC_FP64)
    rc = gp_gram_fp64(ctx);
  else
    rc = gp_gram_split(ctx, opts->precision);
  if (rc) return rc;
  GP_CUDA(ctx, cudaEventRecord(ctx->ev_g1, ctx->stream));

  double *d_tr;
  rc = gp_scratch(ctx, sizeof(double), (void **)&d_tr);
  if (rc) return rc;
  rc = gp_launch_symmetrize_trace(ctx, d_tr);
  if (rc) return rc;
  double tr = 0.0;
  GP_CUDA(ctx, gp_memcpy(ctx, &tr, d_tr, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (n0 || n1 || nmiss) {
    std::vector<int32_t> cnt((size_t)nc * 3);
    GP_CUDA(ctx, gp_memcpy(ctx, cnt.data(), ctx->d_cnt, sizeof(int32_t) * cnt.size(),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int32_t c = 0; c < nc; ++c) {
      if (n0) n0[c] = cnt[3 * (size_t)c];
      if (n1) n1[c] = cnt[3 * (size_t)c + 1];
      if (nmiss) nmiss[c] = cnt[3 * (size_t)c + 2];
    }
  }
  if (killed) memcpy(killed, hk.data(), (size_t)nc);
  if (xmean)
    GP_CUDA(ctx, gp_memcpy(ctx, xmean, ctx->d_xmean, sizeof(double) * nc,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  if (xfancy)
    GP_CUDA(ctx, gp_memcpy(ctx, xfancy, ctx->d_xfancy, sizeof(double) * nc,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  if (XTX)
    GP_CUDA(ctx, gp_memcpy(ctx, XTX, ctx->d_xtx, sizeof(double) * (size_t)need,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  float gms = 0.f;
  GP_CUDA(ctx, cudaEventElapsedTime(&gms, ctx->ev_g0, ctx->ev_g1));
  ctx->gram_ms = gms;
  ctx->gram_flops = (double)n * (double)(n + 1) * (double)ctx->nkept;
  ctx->trace = tr;
  if (trace) *trace = tr;
  if (nused) *nused = ctx->nkept;
  ctx->xtx_valid = 1;
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */

/* evecs[j*n + i] = A[(n-1-j)*n + i]: the top nvec eigenvectors (columns) in descending order */
__global__ void k_take_top(double *evecs, const double *A, int32_t n, int32_t nvec)
{
  int64_t total = (int64_t)n * nvec;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = idx / n, i = idx - j * n;
    evecs[idx] = A[(int64_t)(n - 1 - j) * n + i];
  }
}

extern "C" int gp_eigvecs(gp_ctx *ctx, int32_t nvec, double *evals, double *evecs)
{
  if (!ctx) return GP_ERR_ARG;
  if (!ctx->xtx_valid) return gp_fail(ctx, GP_ERR_STATE, "gp_eigvecs: no Gram (call gp_xtx)");
  const int32_t n = ctx->nrows;
  if (nvec < 0 || nvec > n) return gp_fail(ctx, GP_ERR_ARG, "gp_eigvecs: nvec %d", nvec);
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  /* y = trace/(n-1); XTX *= 1/y  (smartpca.c:1230-1236) */
  double y = ctx->trace / (double)(n - 1);
  if (isnan(y)) return gp_fail(ctx, GP_ERR_NODATA, "bad XTX matrix");
  if (y <= 0.0) return gp_fail(ctx, GP_ERR_NODATA, "XTX has zero trace (perhaps no data)");
  int64_t nn = (int64_t)n * n;
  int blocks = (int)((nn + 255) / 256);
  if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
  k_scale<<<blocks, 256, 0, ctx->stream>>>(ctx->d_xtx, nn, 1.0 / y);
  GP_LAUNCH_CHECK(ctx, "k_scale");
  ctx->keep_valid = 0;
  if (ctx->keep_gram) {
    /* the scaled Gram for the relatedness scan (the eigensolve overwrites d_xtx) */
    if (ctx->keep_cap < nn) {
      if (ctx->d_xtx_keep) cudaFree(ctx->d_xtx_keep);
      ctx->d_xtx_keep = NULL;
      ctx->keep_cap = 0;
      GP_CUDA(ctx, cudaMalloc((void **)&ctx->d_xtx_keep, sizeof(double) * (size_t)nn));
      ctx->keep_cap = nn;
    }
    GP_CUDA(ctx, cudaMemcpyAsync(ctx->d_xtx_keep, ctx->d_xtx, sizeof(double) * (size_t)nn,
                                 cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->keep_valid = 1;
  }

  int rc = gp_realloc(ctx, (void **)&ctx->d_evals, sizeof(double) * (size_t)n);
  if (rc) return rc;
  int32_t keep = nvec > 0 ? nvec : 1;
  rc = gp_realloc(ctx, (void **)&ctx->d_evecs, sizeof(double) * (size_t)n * keep);
  if (rc) return rc;
  const char *alt = getenv("GP_EIG_SYEVD");
  if (!(alt && alt[0] == '1')) {
    /* tridiagonalisation + bisection + inverse iteration for the top vectors (gp_eig.cu) */
    rc = gp_eig_tridiag(ctx, n, nvec, ctx->d_evals, ctx->d_evecs);
    if (rc) return rc;
    if (evals)
      GP_CUDA(ctx, gp_memcpy(ctx, evals, ctx->d_evals, sizeof(double) * (size_t)n,
                             cudaMemcpyDeviceToHost, ctx->stream));
    if (evecs && nvec > 0)
      GP_CUDA(ctx, gp_memcpy(ctx, evecs, ctx->d_evecs, sizeof(double) * (size_t)n * nvec,
                             cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->xtx_valid = 0; /* sytrd overwrote the Gram */
  } else {
    int lwork = 0;
    if (cusolverDnDsyevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                    n, ctx->d_xtx, n, ctx->d_evals, &lwork) !=
        CUSOLVER_STATUS_SUCCESS)
      return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDsyevd_bufferSize failed");
    uint8_t *ws;
    rc = gp_scratch(ctx, sizeof(double) * (size_t)lwork + 256, (void **)&ws);
    if (rc) return rc;
    int *d_info = (int *)(ws + sizeof(double) * (size_t)lwork);
    if (cusolverDnDsyevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                         ctx->d_xtx, n, ctx->d_evals, (double *)ws, lwork,
                         d_info) != CUSOLVER_STATUS_SUCCESS)
      return gp_fail(ctx, GP_ERR_SOLVER, "cusolverDnDsyevd failed to launch");
    int info = 0;
    GP_CUDA(ctx, gp_memcpy(ctx, &info, d_info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    if (nvec > 0) {
      int64_t tot = (int64_t)n * nvec;
      int b2 = (int)((tot + 255) / 256);
      if (b2 > ctx->num_sms * 16) b2 = ctx->num_sms * 16;
      k_take_top<<<b2, 256, 0, ctx->stream>>>(ctx->d_evecs, ctx->d_xtx, n, nvec);
      GP_LAUNCH_CHECK(ctx, "k_take_top");
    }
    std::vector<double> w((size_t)n);
    GP_CUDA(ctx, gp_memcpy(ctx, w.data(), ctx->d_evals, sizeof(double) * (size_t)n,
                                 cudaMemcpyDeviceToHost, ctx->stream));
    if (evecs && nvec > 0)
      GP_CUDA(ctx, gp_memcpy(ctx, evecs, ctx->d_evecs, sizeof(double) * (size_t)n * nvec,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->xtx_valid = 0; /* the solver overwrote the Gram with eigenvectors */
    if (info != 0) return gp_fail(ctx, GP_ERR_SOLVER, "eigensolver info = %d", info);
    if (evals)
      for (int32_t i = 0; i < n; ++i) evals[i] = w[(size_t)(n - 1 - i)];
    /* the resident eigenvalues descending, as the tridiagonal path leaves them */
    for (int32_t i = 0; i < n / 2; ++i) std::swap(w[(size_t)i], w[(size_t)(n - 1 - i)]);
    GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_evals, w.data(), sizeof(double) * (size_t)n,
                           cudaMemcpyHostToDevice, ctx->stream));
  }
  ctx->nvec = nvec;
  ctx->eig_valid = 1;
  ctx->weights_valid = 0;
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */
/*
 * Relatedness of smartrel (src/eigensrc/smartrel.c:578-615): from the scaled Gram of the last
 * pass, R = XTX - sum_{i < K} w_i w_i^T with w_i = sqrt(lambda_i) v_i (subouter, in order),
 * then for rows a < b: y = R_ab / sqrt(R_aa R_bb) + 1/(n-1); pairs with y >= relthresh.
 * Same operation order as the reference, every product and sum rounded on its own.
 */
__global__ void k_rel_weights(const double *evals, const double *evecs, int32_t n, int32_t K,
                              double *w)
{
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)K * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = (int32_t)(idx / n);
    w[idx] = __dmul_rn(evecs[idx], __dsqrt_rn(evals[i]));
  }
}

__device__ __forceinline__ double rel_entry(const double *X, const double *w, int32_t n, int32_t K,
                                            int32_t a, int32_t b)
{
  double r = X[(int64_t)a * n + b];
  for (int32_t i = 0; i < K; ++i)
    r = __dsub_rn(r, __dmul_rn(w[(int64_t)i * n + a], w[(int64_t)i * n + b]));
  return r;
}

/* R_aa for every row, once (the scan reads it for both ends of each pair) */
__global__ void k_rel_diag(const double *X, const double *w, int32_t n, int32_t K, double *d)
{
  for (int32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x)
    d[a] = rel_entry(X, w, n, K, a, a);
}

__global__ void k_rel_scan(const double *X, const double *w, const double *d, int32_t n,
                           int32_t K, double relthresh, int64_t max_pairs, int32_t *pa,
                           int32_t *pb, double *ps, unsigned long long *count)
{
  const int64_t total = (int64_t)n * (n - 1) / 2;
  const double add = 1.0 / (double)(n - 1);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    /* t -> (a, b), a < b, row by row of the strict upper triangle */
    int32_t a = (int32_t)floor(((2.0 * n - 1.0) - sqrt((2.0 * n - 1.0) * (2.0 * n - 1.0) - 8.0 * (double)t)) * 0.5);
    while (a > 0 && (int64_t)a * (2 * (int64_t)n - a - 1) / 2 > t) --a;
    while ((int64_t)(a + 1) * (2 * (int64_t)n - a - 2) / 2 <= t) ++a;
    const int32_t b = (int32_t)(t - (int64_t)a * (2 * (int64_t)n - a - 1) / 2) + a + 1;
    const double y1 = d[a], y2 = d[b];
    const double y = __dadd_rn(__ddiv_rn(rel_entry(X, w, n, K, a, b), __dsqrt_rn(__dmul_rn(y1, y2))), add);
    if (y < relthresh) continue;
    const unsigned long long slot = atomicAdd(count, 1ull);
    if ((int64_t)slot < max_pairs) {
      pa[slot] = a;
      pb[slot] = b;
      ps[slot] = y;
    }
  }
}

extern "C" int gp_keep_gram(gp_ctx *ctx, int32_t keep)
{
  if (!ctx) return GP_ERR_ARG;
  ctx->keep_gram = keep ? 1 : 0;
  return GP_OK;
}

extern "C" int gp_relate(gp_ctx *ctx, int32_t numeigs, double relthresh, int64_t max_pairs,
                         int32_t *pair_a, int32_t *pair_b, double *score, int64_t *npairs)
{
  if (!ctx || !npairs || max_pairs < 0 || (max_pairs > 0 && (!pair_a || !pair_b || !score)))
    return GP_ERR_ARG;
  if (!ctx->keep_valid || !ctx->eig_valid)
    return gp_fail(ctx, GP_ERR_STATE, "gp_relate: no kept Gram (gp_keep_gram before gp_eigvecs)");
  const int32_t n = ctx->nrows, K = numeigs;
  if (K < 0 || K > ctx->nvec) return gp_fail(ctx, GP_ERR_ARG, "gp_relate: numeigs %d > %d", K, ctx->nvec);
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t nw = (size_t)K * n;
  size_t bytes = sizeof(double) * (nw + (size_t)n + (size_t)max_pairs) +
                 sizeof(int32_t) * 2 * (size_t)max_pairs + 1024;
  uint8_t *base;
  int rc = gp_scratch(ctx, bytes, (void **)&base);
  if (rc) return rc;
  double *d_w = (double *)base, *d_d = d_w + nw, *d_s = d_d + n;
  int32_t *d_a = (int32_t *)(d_s + max_pairs), *d_b = d_a + max_pairs;
  unsigned long long *d_cnt = (unsigned long long *)(((uintptr_t)(d_b + max_pairs) + 15) & ~(uintptr_t)15);
  GP_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), ctx->stream));
  if (nw) {
    int blocks = (int)((nw + 255) / 256);
    if (blocks > ctx->num_sms * 8) blocks = ctx->num_sms * 8;
    k_rel_weights<<<blocks, 256, 0, ctx->stream>>>(ctx->d_evals, ctx->d_evecs, n, K, d_w);
    GP_LAUNCH_CHECK(ctx, "k_rel_weights");
  }
  if (n > 1) {
    k_rel_diag<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->d_xtx_keep, d_w, n, K, d_d);
    GP_LAUNCH_CHECK(ctx, "k_rel_diag");
    k_rel_scan<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(ctx->d_xtx_keep, d_w, d_d, n, K,
                                                          relthresh, max_pairs, d_a, d_b, d_s,
                                                          d_cnt);
    GP_LAUNCH_CHECK(ctx, "k_rel_scan");
  }
  unsigned long long cnt = 0;
  GP_CUDA(ctx, gp_memcpy(ctx, &cnt, d_cnt, sizeof cnt, cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *npairs = (int64_t)cnt;
  const int64_t got = (int64_t)cnt < max_pairs ? (int64_t)cnt : max_pairs;
  if (got > 0) {
    GP_CUDA(ctx, gp_memcpy(ctx, pair_a, d_a, sizeof(int32_t) * (size_t)got, cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, gp_memcpy(ctx, pair_b, d_b, sizeof(int32_t) * (size_t)got, cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, gp_memcpy(ctx, score, d_s, sizeof(double) * (size_t)got, cudaMemcpyDeviceToHost, ctx->stream));
    GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */

extern "C" int gp_ridoutlier(const double *evecs, int32_t n, int32_t neigs, double thresh,
                             int32_t mode, int32_t *badlist, int32_t *vecno, double *score)
{
  /* restates ridoutlier (src/eigensrc/smartsubs.c:18-91) with the same operation order */
  if (!evecs || !badlist || n < 0 || neigs < 0) return GP_ERR_ARG;
  if (mode > 1) return 0;
  if (n < 3) return 0;
  std::vector<double> ww((size_t)n), w2((size_t)n);
  std::vector<int> vbad((size_t)n, 0), vno((size_t)n, -1);
  std::vector<double> sc((size_t)n, 0.0);
  for (int32_t i = 0; i < neigs; ++i) {
    memcpy(ww.data(), evecs + (size_t)i * n, sizeof(double) * (size_t)n);
    if (mode == 0) {
      double y1 = 0.0;
      for (int32_t j = 0; j < n; ++j) y1 += ww[(size_t)j];
      y1 = y1 / (double)n;
      for (int32_t j = 0; j < n; ++j) ww[(size_t)j] = ww[(size_t)j] + (-y1);
      double y2 = 0.0;
      for (int32_t j = 0; j < n; ++j) y2 += ww[(size_t)j] * ww[(size_t)j];
      y2 = y2 / (double)n;
      y2 = sqrt(y2);
      double inv = 1.0 / y2;
      for (int32_t j = 0; j < n; ++j) ww[(size_t)j] = ww[(size_t)j] * inv;
      for (int32_t j = 0; j < n; ++j) {
        if (fabs(ww[(size_t)j]) > thresh) {
          vbad[(size_t)j] = 1;
          if (vno[(size_t)j] < 0) {
            vno[(size_t)j] = i;
            sc[(size_t)j] = ww[(size_t)j];
          }
        }
      }
    } else {
      for (int32_t j = 0; j < n; ++j) {
        double yy = ww[(size_t)j];
        ww[(size_t)j] = 0;
        double y1 = 0.0;
        for (int32_t t = 0; t < n; ++t) y1 += ww[(size_t)t];
        y1 = y1 / (double)(n - 1);
        for (int32_t t = 0; t < n; ++t) w2[(size_t)t] = ww[(size_t)t] + (-y1);
        w2[(size_t)j] = 0;
        double y2 = 0.0;
        for (int32_t t = 0; t < n; ++t) y2 += w2[(size_t)t] * w2[(size_t)t];
        y2 = y2 / (double)n;
        y2 = sqrt(y2);
        double zz = yy - y1;
        zz /= y2;
        if (fabs(zz) > thresh) {
          vbad[(size_t)j] = 1;
          if (vno[(size_t)j] < 0) {
            vno[(size_t)j] = i;
            sc[(size_t)j] = zz;
          }
        }
        ww[(size_t)j] = yy;
      }
    }
  }
  int32_t nbad = 0;
  for (int32_t j = 0; j < n; ++j) {
    if (vecno) vecno[j] = vno[(size_t)j];
    if (score) score[j] = sc[(size_t)j];
    if (vbad[(size_t)j] == 1) badlist[nbad++] = j;
  }
  return nbad;
}

/* ------------------------------------------------------------------------------------ */

/* B[r*K + j] = 10 * evecs[j*n + r]   (setfvecs src/qpsubs.c:489-507) */
__global__ void k_fvecs_T(double *B, const double *evecs, int32_t n, int32_t K)
{
  int64_t total = (int64_t)n * K;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = idx / K, j = idx - r * K;
    B[idx] = evecs[j * n + r] * 10.0;
  }
}

/* per kept column: record index, value table (vtab) and the fixxrow table
 * r(g) = g*fancy - xmean (src/qpsubs.c:338-348), missing -> 0 */
__global__ void k_kept_tables(const int32_t *kept, int32_t nkept, const int32_t *cols,
                              const double *vtab, const double *xmean, const double *xfancy,
                              int32_t *snprec, double *vt, double *rt, double *ot)
{
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nkept; k += gridDim.x * blockDim.x) {
    int32_t c = kept[k];
    snprec[k] = cols[c];
    for (int t = 0; t < 4; ++t) vt[4 * k + t] = vtab[4 * c + t];
    double f = xfancy[c], m = xmean[c];
    for (int g = 0; g < 3; ++g) {
      double x = __dmul_rn((double)g, f);
      rt[4 * k + g] = (x < -0.001) ? 0.0 : __dsub_rn(x, m);
    }
    rt[4 * k + 3] = 0.0;
    ot[4 * k] = ot[4 * k + 1] = ot[4 * k + 2] = 1.0;
    ot[4 * k + 3] = 0.0;
  }
}

/* ffvT[k][j] = fancy_c Yg[k][j] - xmean_c Yo[k][j], c = kept[k]  (X = G fancy - O xmean) */
__global__ void k_combine_gx(double *ffvT, const double *yg, const double *yo, const int32_t *kept,
                             const double *xfancy, const double *xmean, int32_t nk, int32_t K)
{
  int64_t total = (int64_t)nk * K;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = kept[idx / K];
    ffvT[idx] = xfancy[c] * yg[idx] - xmean[c] * yo[idx];
  }
}

/* a[k][j] = fancy_c w[k][j], b[k][j] = xmean_c w[k][j], c = kept[k] */
__global__ void k_scale_rows2(double *a, double *b, const double *w, const int32_t *kept,
                              const double *xfancy, const double *xmean, int32_t nk, int32_t K)
{
  int64_t total = (int64_t)nk * K;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = kept[idx / K];
    a[idx] = xfancy[c] * w[idx];
    b[idx] = xmean[c] * w[idx];
  }
}

/* ffvecs[j*ncols + kept[k]] = ffvT[k*K + j] (killed columns stay 0) */
__global__ void k_scatter_ffvecs(double *ffvecs, const double *ffvT, const int32_t *kept,
                                 int32_t nkept, int32_t ncols, int32_t K)
{
  int64_t total = (int64_t)nkept * K;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t k = idx / K, j = idx - k * K;
    ffvecs[j * ncols + kept[k]] = ffvT[idx];
  }
}

struct kept_tables {
  int32_t *snprec;
  double *vt, *rt, *ot;
};

static int build_kept_tables(gp_ctx *ctx, uint8_t *base, kept_tables *t)
{
  int32_t nk = ctx->nkept;
  t->vt = (double *)base;
  t->rt = t->vt + 4 * (size_t)nk;
  t->ot = t->rt + 4 * (size_t)nk;
  t->snprec = (int32_t *)(t->ot + 4 * (size_t)nk);
  if (nk == 0) return GP_OK;
  int blocks = (nk + 255) / 256;
  if (blocks > ctx->num_sms * 8) blocks = ctx->num_sms * 8;
  k_kept_tables<<<blocks, 256, 0, ctx->stream>>>(ctx->d_kept, nk, ctx->d_cols, ctx->d_vtab,
                                                 ctx->d_xmean, ctx->d_xfancy, t->snprec, t->vt,
                                                 t->rt, t->ot);
  GP_LAUNCH_CHECK(ctx, "k_kept_tables");
  return GP_OK;
}

/* bytes of the kept-column tables, rounded up so that what follows stays 256-byte aligned */
static size_t kept_tables_bytes(int32_t nk)
{
  size_t b = (size_t)nk * (12 * sizeof(double) + sizeof(int32_t)) + 256;
  return (b + 255) / 256 * 256;
}

extern "C" int gp_snp_weights(gp_ctx *ctx, int32_t numeigs, double *ffvecs, double *fxvecs,
                              double *fxscal)
{
  if (!ctx || !fxscal) return GP_ERR_ARG;
  if (!ctx->eig_valid) return gp_fail(ctx, GP_ERR_STATE, "gp_snp_weights: call gp_eigvecs first");
  if (numeigs < 1 || numeigs > ctx->nvec)
    return gp_fail(ctx, GP_ERR_ARG, "gp_snp_weights: numeigs %d > resident vectors %d", numeigs,
                   ctx->nvec);
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  const int32_t n = ctx->nrows, nc = ctx->ncols, nk = ctx->nkept, K = numeigs;
  int rc = gp_realloc(ctx, (void **)&ctx->d_ffvecs, sizeof(double) * (size_t)K * nc);
  if (!rc) rc = gp_realloc(ctx, (void **)&ctx->d_fxscal, sizeof(double) * (size_t)K);
  if (rc) return rc;
  size_t off_tab = kept_tables_bytes(nk);
  size_t bytes = off_tab + sizeof(double) * ((size_t)n * K + (size_t)nk * K + (size_t)n * K) + 256;
  uint8_t *base;
  rc = gp_scratch(ctx, bytes, (void **)&base);
  if (rc) return rc;
  kept_tables kt;
  rc = build_kept_tables(ctx, base, &kt);
  if (rc) return rc;
  double *d_B = (double *)(base + off_tab);
  double *d_ffvT = d_B + (size_t)n * K;
  double *d_fxT = d_ffvT + (size_t)nk * K;
  int blocks = (int)(((int64_t)n * K + 255) / 256);
  if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
  k_fvecs_T<<<blocks, 256, 0, ctx->stream>>>(d_B, ctx->d_evecs, n, K);
  GP_LAUNCH_CHECK(ctx, "k_fvecs_T");
  if (ctx->precision != GP_PREC_FP64 && nk > 0) {
    /* tensor-core exact products: X = G fancy - O xmean, so
     * ffvecs^T = fancy (G^T W) - xmean (O^T W) with W = 10 evecs^T over the rows */
    double *tmp;
    rc = gp_scratch_aux(ctx, sizeof(double) * 2 * (size_t)nk * K, (void **)&tmp);
    if (rc) return rc;
    double *d_yg = tmp, *d_yo = tmp + (size_t)nk * K;
    gp_tc_codes A;
    rc = gp_tc_codes_for(ctx, 0, ctx->d_rows, n, kt.snprec, nk, &A);
    if (rc) return rc;
    gp_tc_panel pw = {d_B, K, 1.0, 1};
    rc = gp_geno_panel_tc_codes(ctx, &A, 1, &pw, K, d_yg, K);
    if (rc) return rc;
    pw.count = 0;
    rc = gp_geno_panel_tc_codes(ctx, &A, 1, &pw, K, d_yo, K);
    if (rc) return rc;
    int b3 = (int)(((int64_t)nk * K + 255) / 256);
    if (b3 > ctx->num_sms * 16) b3 = ctx->num_sms * 16;
    k_combine_gx<<<b3, 256, 0, ctx->stream>>>(d_ffvT, d_yg, d_yo, ctx->d_kept, ctx->d_xfancy,
                                             ctx->d_xmean, nk, K);
    GP_LAUNCH_CHECK(ctx, "k_combine_gx");
  } else {
    /* ffvecs^T[k][j] = sum_r v(r,k) * 10 evec_j[r] */
    rc = gp_geno_gemm_f64(ctx, 0, ctx->d_rows, n, kt.snprec, kt.vt, nk, d_B, K, K, d_ffvT, K);
    if (rc) return rc;
  }
  GP_CUDA(ctx, cudaMemsetAsync(ctx->d_ffvecs, 0, sizeof(double) * (size_t)K * nc, ctx->stream));
  if (nk) {
    int b2 = (int)(((int64_t)nk * K + 255) / 256);
    if (b2 > ctx->num_sms * 16) b2 = ctx->num_sms * 16;
    k_scatter_ffvecs<<<b2, 256, 0, ctx->stream>>>(ctx->d_ffvecs, d_ffvT, ctx->d_kept, nk, nc, K);
    GP_LAUNCH_CHECK(ctx, "k_scatter_ffvecs");
  }
  /* fxvecs^T[i][j] = xrow_i . ffvecs_j  (fixxrow values g fancy - xmean) */
  if (ctx->precision != GP_PREC_FP64 && nk > 0) {
    double *tmp;
    rc = gp_scratch_aux(ctx, sizeof(double) * 2 * (size_t)nk * K, (void **)&tmp);
    if (rc) return rc;
    int b3 = (int)(((int64_t)nk * K + 255) / 256);
    if (b3 > ctx->num_sms * 16) b3 = ctx->num_sms * 16;
    k_scale_rows2<<<b3, 256, 0, ctx->stream>>>(tmp, tmp + (size_t)nk * K, d_ffvT, ctx->d_kept,
                                              ctx->d_xfancy, ctx->d_xmean, nk, K);
    GP_LAUNCH_CHECK(ctx, "k_scale_rows2");
    gp_tc_panel pr[2] = {{tmp, K, 1.0, 1}, {tmp + (size_t)nk * K, K, -1.0, 0}};
    rc = gp_geno_panel_tc(ctx, 1, ctx->d_rows, n, kt.snprec, nk, 2, pr, K, d_fxT, K);
    if (rc) return rc;
  } else {
    rc = gp_geno_gemm_f64(ctx, 1, ctx->d_rows, n, kt.snprec, kt.rt, nk, d_ffvT, K, K, d_fxT, K);
    if (rc) return rc;
  }
  std::vector<double> fx((size_t)n * K);
  GP_CUDA(ctx, gp_memcpy(ctx, fx.data(), d_fxT, sizeof(double) * fx.size(),
                               cudaMemcpyDeviceToHost, ctx->stream));
  if (ffvecs)
    GP_CUDA(ctx, gp_memcpy(ctx, ffvecs, ctx->d_ffvecs, sizeof(double) * (size_t)K * nc,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  /* fxscal_j = 1/sqrt(sum_i fxvecs^2) in row order (smartpca.c:1504-1525) */
  for (int32_t j = 0; j < K; ++j) {
    double s = 0.0;
    for (int32_t i = 0; i < n; ++i) {
      double y = fx[(size_t)i * K + j];
      if (fxvecs) fxvecs[(size_t)j * n + i] = y;
      s += y * y;
    }
    fxscal[j] = 1.0 / sqrt(s);
  }
  GP_CUDA(ctx, gp_memcpy(ctx, ctx->d_fxscal, fxscal, sizeof(double) * K, cudaMemcpyHostToDevice,
                               ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->nweights = K;
  ctx->weights_valid = 1;
  return GP_OK;
}

/* ------------------------------------------------------------------------------------ */

/* E[k*K + j] = fxscal_j * ffvecs_j[kept k];  P[k*ldp + pair(a,b)] = E_a E_b (a<=b), then 1 */
/* E[k][j] = fxscal_j ffvecs_j(kept k) and P[k] = (E_a E_b for a <= b in row order, 1):
 * a warp per kept SNP, E of the SNP in shared memory, the pair products written as
 * consecutive doubles (coalesced) from a pair-index table; K <= 64 */
#define EP_THREADS 256
__global__ void __launch_bounds__(EP_THREADS)
k_build_EP(const double *ffvecs, const double *fxscal, const int32_t *kept, int32_t nkept,
           int32_t ncols, int32_t K, double *E, double *P, int32_t ldp)
{
  __shared__ uint8_t pa[64 * 65 / 2], pb[64 * 65 / 2];
  __shared__ double se[EP_THREADS / 32][64];
  const int npair = K * (K + 1) / 2;
  for (int t = threadIdx.x; t < npair; t += blockDim.x) {
    int a = 0, rem = t;
    while (rem >= K - a) {
      rem -= K - a;
      ++a;
    }
    pa[t] = (uint8_t)a;
    pb[t] = (uint8_t)(a + rem);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; k < nkept; k += nw) {
    const int32_t c = kept[k];
    for (int j = lane; j < K; j += 32) {
      const double v = fxscal[j] * ffvecs[(int64_t)j * ncols + c];
      se[warp][j] = v;
      E[k * K + j] = v;
    }
    __syncwarp();
    double *p = P + k * ldp;
    for (int t = lane; t < npair; t += 32) p[t] = se[warp][pa[t]] * se[warp][pb[t]];
    if (lane == 0) p[npair] = 1.0;
    __syncwarp();
  }
}

/*
 * Per sample: assemble co (K x K) from the pair sums, check NaN, Cholesky (choldc
 * src/nicksrc/linsubs.c:361-380) and the two triangular solves (cholsl :331-358), with the
 * reference's loop order and no contraction.  One thread per sample.
 */
__global__ void k_lsq_solve(const double *co, int32_t ldco, const double *rr, int32_t K,
                            int32_t nproj, double *acoef, double *bcoef, int32_t *nobs,
                            int32_t *status, double *work, const int32_t *d_nproj)
{
  if (d_nproj) nproj = *d_nproj; /* a device-resident loop's batch size */
  for (int32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nproj;
       q += gridDim.x * blockDim.x) {
    double *a = work + (int64_t)q * (K * K + 2 * K);
    double *p = a + K * K, *x = p + K;
    const double *cq = co + (int64_t)q * ldco;
    const double *rq = rr + (int64_t)q * K;
    int32_t nob = (int32_t)llrint(cq[K * (K + 1) / 2]);
    nobs[q] = nob;
    for (int j = 0; j < K; ++j) bcoef[(int64_t)j * nproj + q] = rq[j];
    if (nob <= K) {
      status[q] = 1;
      continue;
    }
    int t = 0, bad = 0;
    for (int i = 0; i < K; ++i)
      for (int j = i; j < K; ++j) {
        double v = cq[t++];
        a[i * K + j] = v;
        a[j * K + i] = v;
        if (isnan(v)) bad = 1;
      }
    for (int j = 0; j < K; ++j)
      if (isnan(rq[j])) bad = 1;
    if (!bad) {
      for (int i = 0; i < K && !bad; ++i) {
        for (int j = i; j < K; ++j) {
          double sum = a[i * K + j];
          for (int k = i - 1; k >= 0; --k) sum = __dsub_rn(sum, __dmul_rn(a[i * K + k], a[j * K + k]));
          if (i == j) {
            if (sum <= 0.0) {
              bad = 1;
              break;
            }
            p[i] = __dsqrt_rn(sum);
          } else {
            a[j * K + i] = __ddiv_rn(sum, p[i]);
          }
        }
      }
    }
    if (bad) {
      status[q] = 2;
      continue;
    }
    for (int i = 0; i < K; ++i) {
      double sum = rq[i];
      for (int k = i - 1; k >= 0; --k) sum = __dsub_rn(sum, __dmul_rn(a[i * K + k], x[k]));
      x[i] = __ddiv_rn(sum, p[i]);
    }
    for (int i = K - 1; i >= 0; --i) {
      double sum = x[i];
      for (int k = i + 1; k < K; ++k) sum = __dsub_rn(sum, __dmul_rn(a[k * K + i], x[k]));
      x[i] = __ddiv_rn(sum, p[i]);
    }
    for (int j = 0; j < K; ++j) acoef[(int64_t)j * nproj + q] = x[j];
    status[q] = 0;
  }
}

static int lsqproj_impl(gp_ctx *ctx, int32_t numeigs, const int32_t *samples,
                        const int32_t *sample_pop, int32_t npop, int32_t nproj, double *acoeffs,
                        double *bcoeffs, int32_t *nobs, int32_t *status)
{
  if (!ctx || !acoeffs || (nproj > 0 && !samples)) return GP_ERR_ARG;
  if (!ctx->weights_valid)
    return gp_fail(ctx, GP_ERR_STATE, "gp_lsqproj: call gp_snp_weights first");
  if (numeigs < 1 || numeigs > ctx->nweights || numeigs > 64)
    return gp_fail(ctx, GP_ERR_ARG, "gp_lsqproj: numeigs %d out of range", numeigs);
  if (nproj == 0) return GP_OK;
  for (int32_t q = 0; q < nproj; ++q)
    if (samples[q] < 0 || samples[q] >= ctx->nind_all)
      return gp_fail(ctx, GP_ERR_ARG, "gp_lsqproj: sample %d out of range", samples[q]);
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  const int32_t K = numeigs, nk = ctx->nkept, nc = ctx->ncols;
  const int32_t npair = K * (K + 1) / 2, ldp = npair + 1;
  size_t off_tab = kept_tables_bytes(nk);
  size_t nE = (size_t)nk * K, nP = (size_t)nk * ldp;
  size_t nco = (size_t)nproj * ldp, nrr = (size_t)nproj * K;
  size_t nwork = (size_t)nproj * (K * K + 2 * K);
  const bool pf = sample_pop != NULL && npop > 0;
  if (pf && ctx->precision != GP_PREC_FP64)
    return gp_fail(ctx, GP_ERR_ARG, "gp_lsqproj_pops: usepopsformissing runs in FP64 precision only");
  if (pf)
    for (int32_t q = 0; q < nproj; ++q)
      if (sample_pop[q] >= npop)
        return gp_fail(ctx, GP_ERR_ARG, "gp_lsqproj_pops: population %d >= npop %d",
                       sample_pop[q], npop);
  const size_t off_fill = pf ? gp_lsq_fill_work_bytes(nproj, nk, npop) : 0;
  size_t bytes = off_tab + sizeof(double) * (nE + nP + nco + nrr + nwork + 2 * nrr) +
                 sizeof(int32_t) * (4 * (size_t)nproj) + off_fill + 1024;
  uint8_t *base;
  int rc = gp_scratch(ctx, bytes, (void **)&base);
  if (rc) return rc;
  kept_tables kt;
  rc = build_kept_tables(ctx, base, &kt);
  if (rc) return rc;
  double *d_E = (double *)(base + off_tab);
  double *d_P = d_E + nE, *d_co = d_P + nP, *d_rr = d_co + nco, *d_work = d_rr + nrr;
  double *d_a = d_work + nwork, *d_b = d_a + nrr;
  int32_t *d_samp = (int32_t *)(d_b + nrr), *d_nobs = d_samp + nproj, *d_st = d_nobs + nproj;
  int32_t *d_spop = d_st + nproj;
  void *fill_work = (void *)((((uintptr_t)(d_spop + nproj)) + 255) & ~(uintptr_t)255);
  GP_CUDA(ctx, gp_memcpy(ctx, d_samp, samples, sizeof(int32_t) * (size_t)nproj,
                               cudaMemcpyHostToDevice, ctx->stream));
  double *d_raw = NULL, *d_of = NULL, *d_rf = NULL;
  if (pf && nk > 0) {
    GP_CUDA(ctx, gp_memcpy(ctx, d_spop, sample_pop, sizeof(int32_t) * (size_t)nproj,
                           cudaMemcpyHostToDevice, ctx->stream));
    rc = gp_lsq_fill_tables(ctx, d_samp, d_spop, nproj, npop, K, kt.snprec, kt.ot, nk,
                            fill_work, &d_raw, &d_of, &d_rf);
    if (rc) return rc;
  }
  if (nk) {
    int blocks = (nk + EP_THREADS / 32 - 1) / (EP_THREADS / 32);
    if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
    k_build_EP<<<blocks, EP_THREADS, 0, ctx->stream>>>(ctx->d_ffvecs, ctx->d_fxscal, ctx->d_kept,
                                                       nk, nc, K, d_E, d_P, ldp);
    GP_LAUNCH_CHECK(ctx, "k_build_EP");
  }
  /* masked normal equations: co = O P (pair sums + observed count), rr = R E */
  if (ctx->precision != GP_PREC_FP64 && nk > 0) {
    gp_tc_codes A;
    /* projecting exactly the analysis rows: the product can reuse their codes */
    const int32_t *d_list = d_samp;
    if (nproj == ctx->nrows && ctx->h_rows &&
        memcmp(samples, ctx->h_rows, sizeof(int32_t) * (size_t)nproj) == 0)
      d_list = ctx->d_rows;
    rc = gp_tc_codes_for(ctx, 1, d_list, nproj, kt.snprec, nk, &A);
    if (rc) return rc;
    gp_tc_panel pc = {d_P, ldp, 1.0, 0};
    rc = gp_geno_panel_tc_codes(ctx, &A, 1, &pc, ldp, d_co, ldp);
    if (rc) return rc;
    double *tmp;
    rc = gp_scratch_aux(ctx, sizeof(double) * 2 * (size_t)nk * K, (void **)&tmp);
    if (rc) return rc;
    int b3 = (int)(((int64_t)nk * K + 255) / 256);
    if (b3 > ctx->num_sms * 16) b3 = ctx->num_sms * 16;
    k_scale_rows2<<<b3, 256, 0, ctx->stream>>>(tmp, tmp + (size_t)nk * K, d_E, ctx->d_kept,
                                              ctx->d_xfancy, ctx->d_xmean, nk, K);
    GP_LAUNCH_CHECK(ctx, "k_scale_rows2");
    gp_tc_panel pr[2] = {{tmp, K, 1.0, 1}, {tmp + (size_t)nk * K, K, -1.0, 0}};
    rc = gp_geno_panel_tc_codes(ctx, &A, 2, pr, K, d_rr, K);
    if (rc) return rc;
  } else if (d_raw) {
    /* usepopsformissing: a filled genotype counts as observed with its fixxrow value */
    rc = gp_geno_gemm_f64_fill(ctx, d_samp, d_spop, nproj, kt.snprec, kt.ot, d_of, npop, nk,
                               d_P, ldp, ldp, d_co, ldp);
    if (rc) return rc;
    rc = gp_geno_gemm_f64_fill(ctx, d_samp, d_spop, nproj, kt.snprec, kt.rt, d_rf, npop, nk,
                               d_E, K, K, d_rr, K);
    if (rc) return rc;
  } else {
    rc = gp_geno_gemm_f64(ctx, 1, d_samp, nproj, kt.snprec, kt.ot, nk, d_P, ldp, ldp, d_co, ldp);
    if (rc) return rc;
    rc = gp_geno_gemm_f64(ctx, 1, d_samp, nproj, kt.snprec, kt.rt, nk, d_E, K, K, d_rr, K);
    if (rc) return rc;
  }
  GP_CUDA(ctx, cudaMemsetAsync(d_a, 0, sizeof(double) * nrr, ctx->stream));
  int blocks = (nproj + 127) / 128;
  k_lsq_solve<<<blocks, 128, 0, ctx->stream>>>(d_co, ldp, d_rr, K, nproj, d_a, d_b, d_nobs, d_st,
                                               d_work, NULL);
  GP_LAUNCH_CHECK(ctx, "k_lsq_solve");
  std::vector<int32_t> st((size_t)nproj);
  std::vector<double> ha(nrr);
  GP_CUDA(ctx, gp_memcpy(ctx, ha.data(), d_a, sizeof(double) * nrr, cudaMemcpyDeviceToHost,
                               ctx->stream));
  GP_CUDA(ctx, gp_memcpy(ctx, st.data(), d_st, sizeof(int32_t) * (size_t)nproj,
                               cudaMemcpyDeviceToHost, ctx->stream));
  if (bcoeffs)
    GP_CUDA(ctx, gp_memcpy(ctx, bcoeffs, d_b, sizeof(double) * nrr, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  std::vector<int32_t> hn((size_t)nproj);
  GP_CUDA(ctx, gp_memcpy(ctx, hn.data(), d_nobs, sizeof(int32_t) * (size_t)nproj,
                         cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<double> raw;
  if (d_raw) {
    raw.resize((size_t)nproj);
    GP_CUDA(ctx, gp_memcpy(ctx, raw.data(), d_raw, sizeof(double) * (size_t)nproj,
                           cudaMemcpyDeviceToHost, ctx->stream));
  }
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int32_t q = 0; q < nproj; ++q) {
    if (d_raw && raw[(size_t)q] <= (double)K) {
      /* the coverage check runs on the observed genotypes, before any fill */
      st[(size_t)q] = 1;
      hn[(size_t)q] = (int32_t)raw[(size_t)q];
      if (bcoeffs)
        for (int32_t j = 0; j < K; ++j) bcoeffs[(size_t)j * nproj + q] = 0.0;
    }
    if (nobs) nobs[q] = hn[(size_t)q];
    if (status) status[q] = st[(size_t)q];
    if (st[(size_t)q] == 2) continue; /* left untouched, as the reference keeps regans */
    for (int32_t j = 0; j < K; ++j)
      acoeffs[(size_t)j * nproj + q] = st[(size_t)q] == 1 ? 0.0 : ha[(size_t)j * nproj + q];
  }
  return GP_OK;
}

extern "C" int gp_lsqproj(gp_ctx *ctx, int32_t numeigs, const int32_t *samples, int32_t nproj,
                          double *acoeffs, double *bcoeffs, int32_t *nobs, int32_t *status)
{
  return lsqproj_impl(ctx, numeigs, samples, NULL, 0, nproj, acoeffs, bcoeffs, nobs, status);
}

extern "C" int gp_lsqproj_pops(gp_ctx *ctx, int32_t numeigs, const int32_t *samples,
                               const int32_t *sample_pop, int32_t npop, int32_t nproj,
                               double *acoeffs, double *bcoeffs, int32_t *nobs, int32_t *status)
{
  if (!sample_pop || npop <= 0)
    return gp_fail(ctx, GP_ERR_ARG, "gp_lsqproj_pops: sample populations are required");
  return lsqproj_impl(ctx, numeigs, samples, sample_pop, npop, nproj, acoeffs, bcoeffs, nobs,
                      status);
}

/* ------------------------------------------------------------------------------------ */

extern "C" int gp_timer_start(gp_ctx *ctx)
{
  if (!ctx) return GP_ERR_ARG;
  GP_CUDA(ctx, cudaEventRecord(ctx->ev_t0, ctx->stream));
  return GP_OK;
}

extern "C" int gp_timer_stop(gp_ctx *ctx, double *ms)
{
  if (!ctx || !ms) return GP_ERR_ARG;
  GP_CUDA(ctx, cudaEventRecord(ctx->ev_t1, ctx->stream));
  GP_CUDA(ctx, cudaEventSynchronize(ctx->ev_t1));
  float f = 0.f;
  GP_CUDA(ctx, cudaEventElapsedTime(&f, ctx->ev_t0, ctx->ev_t1));
  *ms = f;
  return GP_OK;
}

extern "C" int gp_last_tridiag_time(const gp_ctx *ctx, double *ms, int32_t *n)
{
  if (!ctx) return GP_ERR_ARG;
  if (ms) *ms = ctx->tridiag_ms;
  if (n) *n = ctx->tridiag_n;
  return GP_OK;
}

extern "C" int gp_last_counts_time(const gp_ctx *ctx, double *ms, int64_t *bytes)
{
  if (!ctx) return GP_ERR_ARG;
  float f = 0.f;
  if (ctx->counts_bytes > 0) {
    if (cudaEventSynchronize(ctx->ev_c1) != cudaSuccess ||
        cudaEventElapsedTime(&f, ctx->ev_c0, ctx->ev_c1) != cudaSuccess)
      return GP_ERR_CUDA;
  }
  if (ms) *ms = f;
  if (bytes) *bytes = ctx->counts_bytes;
  return GP_OK;
}

extern "C" int gp_last_gram_time(const gp_ctx *ctx, double *ms, int32_t *launches, double *flops)
{
  if (!ctx) return GP_ERR_ARG;
  if (ms) *ms = ctx->gram_ms;
  if (launches) *launches = ctx->gram_launches;
  if (flops) *flops = ctx->gram_flops;
  return GP_OK;
}

extern "C" int gp_host_register(void *ptr, size_t bytes)
{
  if (!ptr || !bytes) return GP_ERR_ARG;
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) return gp_fail(NULL, GP_ERR_CUDA, "cudaHostRegister: %s", cudaGetErrorString(e));
  return GP_OK;
}

extern "C" int gp_host_unregister(void *ptr)
{
  if (!ptr) return GP_ERR_ARG;
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) return gp_fail(NULL, GP_ERR_CUDA, "cudaHostUnregister: %s", cudaGetErrorString(e));
  return GP_OK;
}

extern "C" int gp_transfer_bytes(gp_ctx *ctx, int64_t *h2d, int64_t *d2h, int32_t reset)
{
  if (!ctx) return GP_ERR_ARG;
  if (h2d) *h2d = ctx->h2d_bytes;
  if (d2h) *d2h = ctx->d2h_bytes;
  if (reset) ctx->h2d_bytes = ctx->d2h_bytes = 0;
  return GP_OK;
}

extern "C" int gp_launch_count(gp_ctx *ctx, int64_t *n, int32_t reset)
{
  if (!ctx) return GP_ERR_ARG;
  if (n) *n = ctx->launches;
  if (reset) ctx->launches = 0;
  return GP_OK;
}
