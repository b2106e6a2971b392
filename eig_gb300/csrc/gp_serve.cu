/*
 * Projection serving on a resident panel (include/gpupca_serve.h): admission by device
 * memory, continuous batching with two batches in flight, exact tensor-core masked normal
 * equations and per-sample FP64 Cholesky solves (the lsqproj/regressit arithmetic of
 * src/eigensrc/smartpca.c:4690-4712 and src/regsubs.c:8-72 restated for a batch).
 */
#include <cuda_runtime.h>
#include <errno.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <deque>
#include <unordered_map>
#include <vector>

#include "../../include/gpupca_run.h"
#include "../../include/gpupca_serve.h"
#include "gp_geno_tc.h"
#include "gp_internal.h"

struct gp_req {
  int64_t id;
  int kind;           /* 0 projection request, 1 full-PCA job */
  /* full-PCA job */
  const gp_panel *panel;
  const gp_smartpca_opts *opts;
  gp_run_result *result;
  int64_t footprint;
  /* projection request */
  int32_t nsamp;
  const uint8_t *codes;
  double *coords;
  int32_t *status;
  int64_t row_start;  /* ring position of the first row */
  int64_t skip;       /* ring rows skipped before it (wrap) */
  cudaEvent_t copied;
  int64_t seq;        /* position in the device loop's queue */
  int done;
  int error;
};

/* The device-resident loop's queue, in mapped pinned host memory.  The host writes request
 * descriptors, then n_pub (release); the loop writes each request's error word, then n_done
 * (release), and its counters. */
#define SRV_QCAP 8192
struct gp_srv_queue {
  int64_t n_pub;
  int64_t n_done;
  int64_t batches;
  int64_t idle_polls;
  int32_t stop;
  int32_t err;
  int64_t req_row[SRV_QCAP];
  int32_t req_n[SRV_QCAP];
  int32_t req_err[SRV_QCAP];
};
#define SRV_POLL_NS 1000000ull /* one poll of the loop waits at most 1 ms for a request */
/* tickets are released by the gp_serve_test / gp_serve_wait call that sees them complete */

struct gp_batch {
  std::vector<gp_req *> reqs;
  int64_t row_start;
  int32_t nrows;
  int slot;
  int failed; /* launch error: its finished event was never recorded */
  cudaEvent_t finished;
};

struct gp_server {
  gp_ctx *ctx;
  int32_t K, npair, ldp, nk;
  std::vector<int32_t> snp_index; /* panel SNP k -> genotype SNP record */
  int64_t row_bytes;
  int32_t max_batch;
  int64_t pool_cap;
  int fp64_serial;
  std::vector<double> eigscale;
  /* resident panel */
  double *d_E, *d_P, *d_fE, *d_mE;
  double *d_otab, *d_rtab;
  void *stor_co, *stor_rr;
  gp_tc_prepared Pco, Prr;
  /* pool and per-slot batch buffers */
  uint8_t *d_pool;
  int64_t head, tail;
  cudaStream_t copy_stream;
  double *d_co[2], *d_rr[2], *d_a[2], *d_b[2], *d_work[2], *d_part[2];
  int32_t *d_nobs[2], *d_status[2];
  int *d_errw[2];
  double *h_a[2];
  int32_t *h_status[2];
  int *h_err[2];
  /* queues */
  pthread_mutex_t mu;
  pthread_cond_t cv;
  std::deque<gp_req *> waiting, admitted;
  std::deque<gp_batch *> inflight;
  std::unordered_map<int64_t, gp_req *> all;
  int64_t next_id;
  /* full-PCA jobs: FIFO, admitted while their footprint fits the budget */
  std::deque<gp_req *> pca_waiting;
  std::vector<gp_ctx *> wctx;
  std::vector<pthread_t> workers;
  int64_t pca_budget, pca_used;
  int32_t pca_running, pca_peak;
  int64_t pca_done;
  pthread_t thread;
  int stop, thread_started, paused;
  int64_t n_batches, n_samples, n_requests;
  /* the device-resident loop */
  int host_loop;
  gp_srv_queue *hq, *dq;      /* host and device views of the queue */
  double *h_res, *d_res;      /* [pool_cap*K] coordinates at the request rows (mapped) */
  int32_t *h_rst, *d_rst;     /* [pool_cap] statuses (mapped) */
  gp_tc_batch *d_batch;
  double *d_Z, *d_escale;
  cudaGraph_t graph;
  cudaGraphExec_t gexec;
  int loop_running;
  int64_t loop_launches, n_pub, n_done_seen;
  std::deque<gp_req *> published;
  char err[GP_ERRLEN];
};

/* FP64 products for the serial baseline: Y[q][c] = sum_s T_s[code(q,s)] P[s][c], codes
 * sample-major (row q at codes + q*ldc); split over s into part[split][q][c] */
#define ST 64
#define SK 16
__global__ void __launch_bounds__(256)
k_codes_gemm_f64(const uint8_t *__restrict__ codes, int64_t ldc, int32_t nrows,
                 const double *__restrict__ tab, int32_t nk, const double *__restrict__ P,
                 int64_t ldp, int32_t ncols, int32_t kper, double *part)
{
  __shared__ double As[SK][ST + 1];
  __shared__ double Bs[SK][ST + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int32_t q0 = (int32_t)blockIdx.y * ST, c0 = (int32_t)blockIdx.x * ST;
  const int32_t kb = (int32_t)blockIdx.z * kper, ke = kb + kper < nk ? kb + kper : nk;
  const int lk = tid & 15, lr = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int32_t k0 = kb; k0 < ke; k0 += SK) {
    int32_t s = k0 + lk;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      int32_t q = q0 + lr + 16 * p;
      double v = 0.0;
      if (s < ke && q < nrows) {
        uint32_t c = (codes[(int64_t)q * ldc + (s >> 2)] >> ((3 - (s & 3)) * 2)) & 3u;
        v = tab[4 * s + c];
      }
      As[lk][lr + 16 * p] = v;
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      int e = tid + 256 * p;
      int r = e >> 6, c = e & 63;
      int32_t ss = k0 + r, cc = c0 + c;
      Bs[r][c] = (ss < ke && cc < ncols) ? P[(int64_t)ss * ldp + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        a[p] = As[k][ty + 16 * p];
        b[p] = Bs[k][tx + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[p][r] = fma(a[p], b[r], acc[p][r]);
    }
    __syncthreads();
  }
  double *o = part + (int64_t)blockIdx.z * nrows * ncols;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    int32_t q = q0 + ty + 16 * p;
    if (q >= nrows) continue;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int32_t c = c0 + tx + 16 * r;
      if (c < ncols) o[(int64_t)q * ncols + c] = acc[p][r];
    }
  }
}

__global__ void k_parts_sum(double *Y, int64_t ldy, const double *part, int32_t nsplit,
                            int32_t nrows, int32_t ncols)
{
  int64_t total = (int64_t)nrows * ncols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = idx / ncols, c = idx - q * ncols;
    double s = 0.0;
    for (int32_t t = 0; t < nsplit; ++t) s += part[t * total + idx];
    Y[q * ldy + c] = s;
  }
}

/* panel arrays of the server from the source handle (kept columns in kept order) */
__global__ void k_serve_panel(const double *ffvecs, const double *fxscal, const int32_t *kept,
                              const double *xfancy, const double *xmean, int32_t nk, int32_t ncols,
                              int32_t K, double *E, double *P, int32_t ldp, double *fE, double *mE,
                              double *otab, double *rtab)
{
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
    int32_t c = kept[k];
    double f = xfancy[c], m = xmean[c];
    double e[64];
    for (int j = 0; j < K; ++j) {
      e[j] = fxscal[j] * ffvecs[(int64_t)j * ncols + c];
      E[(int64_t)k * K + j] = e[j];
      fE[(int64_t)k * K + j] = f * e[j];
      mE[(int64_t)k * K + j] = m * e[j];
    }
    double *p = P + (int64_t)k * ldp;
    int t = 0;
    for (int a = 0; a < K; ++a)
      for (int b = a; b < K; ++b) p[t++] = e[a] * e[b];
    p[t] = 1.0;
    otab[4 * k] = otab[4 * k + 1] = otab[4 * k + 2] = 1.0;
    otab[4 * k + 3] = 0.0;
    for (int g = 0; g < 3; ++g) {
      double x = __dmul_rn((double)g, f);
      rtab[4 * k + g] = (x < -0.001) ? 0.0 : __dsub_rn(x, m);
    }
    rtab[4 * k + 3] = 0.0;
  }
}

/* ---- the device-resident loop's kernels -------------------------------------------- */

__device__ __forceinline__ uint64_t srv_globaltimer()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int64_t ld_acquire_sys(const int64_t *p)
{
  int64_t v;
  asm volatile("ld.acquire.sys.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_sys(int64_t *p, int64_t v)
{
  asm volatile("st.release.sys.global.s64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

/*
 * The loop's batch former (one thread): waits, at most poll_ns, for requests published
 * beyond those taken, then packs the published requests whose rows follow one another in
 * the pool, up to max_batch rows, into the next batch.  Sets the loop's condition: 0 when the
 * host asked it to stop and nothing is left, else 1 (an empty batch when the poll ran out).
 */
__global__ void k_srv_take(gp_srv_queue *q, gp_tc_batch *db, const uint8_t *pool,
                           int64_t row_bytes, int32_t max_batch, cudaGraphConditionalHandle h,
                           uint64_t poll_ns)
{
  if (threadIdx.x != 0) return;
  const int64_t taken = db->req_end;
  const uint64_t t0 = srv_globaltimer();
  int64_t pub = ld_acquire_sys(&q->n_pub);
  while (pub <= taken) {
    const bool stop = *(volatile int32_t *)&q->stop != 0;
    if (stop || srv_globaltimer() - t0 > poll_ns) {
      db->nrows = 0;
      db->req_begin = taken;
      if (!stop) *(volatile int64_t *)&q->idle_polls = *(volatile int64_t *)&q->idle_polls + 1;
      cudaGraphSetConditional(h, stop ? 0u : 1u);
      return;
    }
    __nanosleep(256);
    pub = ld_acquire_sys(&q->n_pub);
  }
  const int64_t row0 = *(volatile int64_t *)&q->req_row[taken % SRV_QCAP];
  int32_t n = 0;
  int64_t r = taken;
  while (r < pub) {
    const int64_t rs = *(volatile int64_t *)&q->req_row[r % SRV_QCAP];
    const int32_t rn = *(volatile int32_t *)&q->req_n[r % SRV_QCAP];
    if (r > taken && (rs != row0 + n || n + rn > max_batch)) break;
    n += rn;
    ++r;
  }
  db->codes = pool + row0 * row_bytes;
  db->nrows = n;
  db->row0 = row0;
  db->req_begin = taken;
  db->req_end = r;
  cudaGraphSetConditional(h, 1u);
}

/* the batch's coordinates (scaled by eigscale) and statuses into the mapped result rows */
__global__ void k_srv_emit(const gp_tc_batch *db, const double *a, const int32_t *st,
                           const double *escale, int32_t K, double *res, int32_t *rst)
{
  const int32_t n = db->nrows;
  const int64_t row0 = db->row0;
  for (int32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int32_t sq = st[q];
    double *o = res + (row0 + q) * K;
    for (int32_t j = 0; j < K; ++j) o[j] = sq == 0 ? a[(int64_t)j * n + q] * escale[j] : 0.0;
    rst[row0 + q] = sq;
  }
  __threadfence_system();
}

/* the batch's error word into its requests, then the completed count (release) */
__global__ void k_srv_done(gp_srv_queue *q, const gp_tc_batch *db, int *err)
{
  if (db->req_end <= db->req_begin) return;
  const int e = *err;
  *err = 0;
  for (int64_t r = db->req_begin; r < db->req_end; ++r) q->req_err[r % SRV_QCAP] = e;
  if (e) q->err = e;
  q->batches = q->batches + 1;
  __threadfence_system();
  st_release_sys(&q->n_done, db->req_end);
}

static int srv_fail(gp_server *s, int code, const char *msg)
{
  snprintf(s->err, sizeof s->err, "%s", msg);
  return code;
}

/* admission by pool memory, in FIFO order; called with the lock held */
static void admit_waiting(gp_server *s)
{
  while (!s->waiting.empty()) {
    gp_req *r = s->waiting.front();
    int64_t used = s->head - s->tail;
    if (used == 0) s->head = s->tail = 0; /* an empty ring restarts at row 0 */
    int64_t pos = s->head % s->pool_cap;
    int64_t skip = (pos + r->nsamp > s->pool_cap) ? s->pool_cap - pos : 0;
    if (used + skip + r->nsamp > s->pool_cap) break; /* waits until memory frees up */
    s->head += skip;
    r->skip = skip;
    r->row_start = s->head % s->pool_cap;
    s->head += r->nsamp;
    cudaError_t e = cudaMemcpyAsync(s->d_pool + r->row_start * s->row_bytes, r->codes,
                                    (size_t)r->nsamp * s->row_bytes, cudaMemcpyHostToDevice,
                                    s->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(r->copied, s->copy_stream);
    if (e != cudaSuccess) r->error = GP_ERR_CUDA;
    s->waiting.pop_front();
    s->admitted.push_back(r);
  }
}

/* queue the batch's work on the compute stream; called without the lock */
static int launch_batch(gp_server *s, gp_batch *b)
{
  gp_ctx *ctx = s->ctx;
  const int sl = b->slot;
  for (gp_req *r : b->reqs) GP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, r->copied, 0));
  GP_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
  gp_tc_codes A;
  A.codes = s->d_pool + b->row_start * s->row_bytes;
  A.ldc = s->row_bytes;
  A.row_map = NULL;
  A.nrows = b->nrows;
  A.k0 = s->nk;
  int rc;
  if (!s->fp64_serial) {
    rc = gp_tc_apply(ctx, &A, &s->Pco, s->d_co[sl], s->ldp, 0);
    if (!rc) rc = gp_tc_apply(ctx, &A, &s->Prr, s->d_rr[sl], s->K, 0);
    if (rc) return rc;
  } else {
    const int32_t n = b->nrows;
    for (int which = 0; which < 2; ++which) {
      const double *P = which ? s->d_E : s->d_P;
      const double *tab = which ? s->d_rtab : s->d_otab;
      int32_t nc = which ? s->K : s->ldp;
      double *Y = which ? s->d_rr[sl] : s->d_co[sl];
      int64_t tiles = (int64_t)((n + ST - 1) / ST) * ((nc + ST - 1) / ST);
      int32_t nsplit = (int32_t)((2 * ctx->num_sms + tiles - 1) / tiles);
      if (nsplit > 16) nsplit = 16;
      if (nsplit < 1) nsplit = 1;
      int32_t kper = ((s->nk + nsplit - 1) / nsplit + SK - 1) / SK * SK;
      nsplit = (s->nk + kper - 1) / kper;
      dim3 grid((unsigned)((nc + ST - 1) / ST), (unsigned)((n + ST - 1) / ST), (unsigned)nsplit);
      k_codes_gemm_f64<<<grid, 256, 0, ctx->stream>>>(A.codes, A.ldc, n, tab, s->nk, P, nc, nc,
                                                       kper, s->d_part[sl]);
      GP_LAUNCH_CHECK(ctx, "k_codes_gemm_f64");
      int64_t tot = (int64_t)n * nc;
      int blocks = (int)((tot + 255) / 256);
      if (blocks > ctx->num_sms * 8) blocks = ctx->num_sms * 8;
      k_parts_sum<<<blocks, 256, 0, ctx->stream>>>(Y, nc, s->d_part[sl], nsplit, n, nc);
      GP_LAUNCH_CHECK(ctx, "k_parts_sum");
    }
  }
  k_lsq_solve<<<(b->nrows + 127) / 128, 128, 0, ctx->stream>>>(
      s->d_co[sl], s->ldp, s->d_rr[sl], s->K, b->nrows, s->d_a[sl], s->d_b[sl], s->d_nobs[sl],
      s->d_status[sl], s->d_work[sl], NULL);
  GP_LAUNCH_CHECK(ctx, "k_lsq_solve");
  GP_CUDA(ctx, cudaMemcpyAsync(s->h_a[sl], s->d_a[sl], sizeof(double) * (size_t)s->K * b->nrows,
                               cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaMemcpyAsync(s->h_status[sl], s->d_status[sl], sizeof(int32_t) * b->nrows,
                               cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaMemcpyAsync(s->h_err[sl], ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GP_CUDA(ctx, cudaEventRecord(b->finished, ctx->stream));
  return GP_OK;
}

/* results of a finished batch into the requests; called with the lock held */
static void complete_batch(gp_server *s, gp_batch *b, int rc)
{
  const int sl = b->slot;
  const int32_t K = s->K, n = b->nrows;
  int err = rc ? rc : (*s->h_err[sl] ? GP_ERR_TIMEOUT : GP_OK);
  int32_t off = 0;
  for (gp_req *r : b->reqs) {
    if (!err && !r->error) {
      for (int32_t q = 0; q < r->nsamp; ++q) {
        int32_t st = s->h_status[sl][off + q];
        r->status[q] = st;
        for (int32_t j = 0; j < K; ++j)
          r->coords[(size_t)q * K + j] =
              st == 0 ? s->h_a[sl][(size_t)j * n + off + q] * s->eigscale[(size_t)j] : 0.0;
      }
    } else if (!r->error) {
      r->error = err;
    }
    off += r->nsamp;
    s->tail += r->skip + r->nsamp;
    cudaEventDestroy(r->copied);
    r->copied = NULL;
    r->done = 1;
    s->n_requests++;
  }
  s->n_batches++;
  s->n_samples += n;
}

/* results of the device loop's completed requests into the callers' buffers; lock held */
static bool complete_published(gp_server *s)
{
  const int64_t done = __atomic_load_n(&s->hq->n_done, __ATOMIC_ACQUIRE);
  s->n_done_seen = done;
  bool any = false;
  const int32_t K = s->K;
  while (!s->published.empty() && s->published.front()->seq < done) {
    gp_req *r = s->published.front();
    s->published.pop_front();
    const int e = s->hq->req_err[r->seq % SRV_QCAP];
    if (!r->error && e) r->error = GP_ERR_TIMEOUT;
    if (!r->error) {
      for (int32_t q = 0; q < r->nsamp; ++q) {
        const int64_t row = r->row_start + q;
        r->status[q] = s->h_rst[row];
        memcpy(r->coords + (size_t)q * K, s->h_res + row * K, sizeof(double) * (size_t)K);
      }
    }
    s->tail += r->skip + r->nsamp;
    cudaEventDestroy(r->copied);
    r->copied = NULL;
    r->done = 1;
    s->n_requests++;
    s->n_samples += r->nsamp;
    any = true;
  }
  s->n_batches = *(volatile int64_t *)&s->hq->batches;
  return any;
}

/* every request still owned by the loop fails with rc (the loop's stream stopped); lock held */
static void fail_loop_requests(gp_server *s, int rc)
{
  for (std::deque<gp_req *> *d : {&s->published, &s->admitted}) {
    for (gp_req *r : *d) {
      if (!r->error) r->error = rc;
      s->tail += r->skip + r->nsamp;
      if (r->copied) cudaEventDestroy(r->copied);
      r->copied = NULL;
      r->done = 1;
    }
    d->clear();
  }
}

/* launch the device-resident loop (lock held); its queue counters carry on from the last run */
static int start_loop(gp_server *s)
{
  __atomic_store_n(&s->hq->stop, 0, __ATOMIC_RELEASE);
  cudaError_t e = cudaGraphLaunch(s->gexec, s->ctx->stream);
  if (e != cudaSuccess) {
    snprintf(s->err, sizeof s->err, "cudaGraphLaunch: %s", cudaGetErrorString(e));
    return GP_ERR_CUDA;
  }
  s->loop_launches++;
  s->loop_running = 1;
  return GP_OK;
}

/* ask the loop to end, wait for it (it drains the published requests and sees the flag
 * within one poll), and hand back what it completed; lock held, released while waiting */
static void stop_loop(gp_server *s)
{
  __atomic_store_n(&s->hq->stop, 1, __ATOMIC_RELEASE);
  pthread_mutex_unlock(&s->mu);
  cudaError_t e = cudaStreamSynchronize(s->ctx->stream);
  pthread_mutex_lock(&s->mu);
  s->loop_running = 0;
  complete_published(s);
  if (e != cudaSuccess || !s->published.empty()) {
    snprintf(s->err, sizeof s->err, "the device-resident serving loop stopped: %s",
             cudaGetErrorString(e));
    fail_loop_requests(s, GP_ERR_CUDA);
  }
  pthread_cond_broadcast(&s->cv);
}

/*
 * The scheduler thread.  With the device-resident loop running it only admits requests into
 * the pool (their copies start on the copy stream), publishes each, in order, once its copy
 * has completed, and hands the loop's results back: it launches nothing.  The loop yields
 * while full-PCA jobs wait or run and while the server is paused (calls that synchronise the
 * whole device, such as cudaFree in a PCA job, would otherwise wait on it); then, and with
 * host_loop or fp64_serial, the thread forms the batches itself and launches each one's
 * kernels, two batches in flight.
 */
static void *scheduler(void *arg)
{
  gp_server *s = (gp_server *)arg;
  cudaSetDevice(s->ctx->device);
  int next_slot = 0;
  pthread_mutex_lock(&s->mu);
  for (;;) {
    admit_waiting(s);
    const bool yield = s->paused || !s->pca_waiting.empty() || s->pca_running > 0;
    if (s->loop_running) {
      if (yield || s->stop) {
        if (s->stop && !yield && (!s->admitted.empty() || !s->waiting.empty())) {
          /* closing: let the loop finish what is queued first */
        } else {
          stop_loop(s);
          continue;
        }
      }
      bool progress = false;
      while (!s->admitted.empty()) {
        gp_req *r = s->admitted.front();
        if (!r->error) {
          cudaError_t q = cudaEventQuery(r->copied);
          if (q == cudaErrorNotReady) break;
          if (q != cudaSuccess) r->error = GP_ERR_CUDA;
        }
        if (s->n_pub - s->n_done_seen >= SRV_QCAP) break;
        const int64_t i = s->n_pub % SRV_QCAP;
        s->hq->req_row[i] = r->row_start;
        s->hq->req_n[i] = r->nsamp;
        r->seq = s->n_pub++;
        __atomic_store_n(&s->hq->n_pub, s->n_pub, __ATOMIC_RELEASE);
        s->admitted.pop_front();
        s->published.push_back(r);
        progress = true;
      }
      if (complete_published(s)) progress = true;
      if (cudaStreamQuery(s->ctx->stream) != cudaErrorNotReady) {
        /* the loop's graph ended without being asked to (a CUDA error) */
        stop_loop(s);
        progress = true;
      }
      if (progress) {
        pthread_cond_broadcast(&s->cv);
        continue;
      }
      if (s->stop && s->waiting.empty() && s->admitted.empty() && s->published.empty()) {
        stop_loop(s);
        continue;
      }
      /* the loop is working on published requests, or a copy is in flight: poll */
      if (!s->published.empty() || !s->admitted.empty()) {
        pthread_mutex_unlock(&s->mu);
        struct timespec ts = {0, 20 * 1000};
        nanosleep(&ts, NULL);
        pthread_mutex_lock(&s->mu);
        continue;
      }
    } else {
      if (s->gexec && !yield && !s->stop && s->inflight.empty()) {
        if (start_loop(s) == GP_OK) continue;
        cudaGraphExecDestroy(s->gexec); /* stay on the host-launched schedule */
        s->gexec = NULL;
      }
      if (!s->paused && s->inflight.size() < 2 && !s->admitted.empty()) {
        /* the next batch: admitted requests, contiguous in the pool, up to max_batch rows */
        gp_batch *b = new gp_batch;
        b->slot = next_slot;
        next_slot ^= 1;
        b->row_start = s->admitted.front()->row_start;
        b->nrows = 0;
        while (!s->admitted.empty()) {
          gp_req *r = s->admitted.front();
          if (!b->reqs.empty() && (s->fp64_serial || r->skip != 0 ||
                                   r->row_start != b->row_start + b->nrows ||
                                   b->nrows + r->nsamp > s->max_batch))
            break;
          b->reqs.push_back(r);
          b->nrows += r->nsamp;
          s->admitted.pop_front();
          if (s->fp64_serial) break;
        }
        b->failed = 0;
        cudaEventCreateWithFlags(&b->finished, cudaEventDisableTiming);
        s->inflight.push_back(b);
        pthread_mutex_unlock(&s->mu);
        int rc = launch_batch(s, b);
        if (rc) {
          /* completes in order behind the batches before it, once the stream has drained */
          cudaStreamSynchronize(s->ctx->stream);
          b->failed = rc;
        }
        pthread_mutex_lock(&s->mu);
        continue;
      }
      if (!s->inflight.empty()) {
        gp_batch *b = s->inflight.front();
        pthread_mutex_unlock(&s->mu);
        cudaError_t e = b->failed ? cudaSuccess : cudaEventSynchronize(b->finished);
        pthread_mutex_lock(&s->mu);
        s->inflight.pop_front();
        complete_batch(s, b, b->failed ? b->failed : (e == cudaSuccess ? GP_OK : GP_ERR_CUDA));
        cudaEventDestroy(b->finished);
        delete b;
        pthread_cond_broadcast(&s->cv);
        continue;
      }
      if (s->stop && s->waiting.empty() && s->admitted.empty()) break;
    }
    struct timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    ts.tv_nsec += 50 * 1000 * 1000;
    if (ts.tv_nsec >= 1000000000L) {
      ts.tv_sec += 1;
      ts.tv_nsec -= 1000000000L;
    }
    pthread_cond_timedwait(&s->cv, &s->mu, &ts);
  }
  pthread_mutex_unlock(&s->mu);
  return NULL;
}

/*
 * The loop: one CUDA graph whose while node runs, per iteration, the batch former, the two
 * exact tensor-core products of the batch's rows (normal equations and right-hand sides),
 * the per-sample solves, the result write-back and the completion count.  Captured once;
 * every kernel reads the batch from d_batch at run time.
 */
static int build_loop(gp_server *s)
{
  gp_ctx *ctx = s->ctx;
  const int32_t K = s->K, mb = s->max_batch;
  cudaGraph_t g = NULL;
  GP_CUDA(ctx, cudaGraphCreate(&g, 0));
  s->graph = g;
  cudaGraphConditionalHandle h;
  GP_CUDA(ctx, cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  GP_CUDA(ctx, cudaGraphAddNode(&node, g, NULL, NULL, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  GP_CUDA(ctx, cudaStreamBeginCaptureToGraph(ctx->stream, body, NULL, NULL, 0,
                                             cudaStreamCaptureModeRelaxed));
  int rc = GP_OK;
  k_srv_take<<<1, 32, 0, ctx->stream>>>(s->dq, s->d_batch, s->d_pool, s->row_bytes, mb, h,
                                       SRV_POLL_NS);
  if (cudaPeekAtLastError() != cudaSuccess) rc = GP_ERR_CUDA;
  if (!rc) rc = gp_tc_apply_dev(ctx, s->d_batch, mb, s->row_bytes, &s->Pco, s->d_Z, s->d_co[0],
                                s->ldp);
  if (!rc) rc = gp_tc_apply_dev(ctx, s->d_batch, mb, s->row_bytes, &s->Prr, s->d_Z, s->d_rr[0], K);
  if (!rc) {
    k_lsq_solve<<<(mb + 127) / 128, 128, 0, ctx->stream>>>(
        s->d_co[0], s->ldp, s->d_rr[0], K, 0, s->d_a[0], s->d_b[0], s->d_nobs[0],
        s->d_status[0], s->d_work[0], &s->d_batch->nrows);
    k_srv_emit<<<(mb + 127) / 128, 128, 0, ctx->stream>>>(s->d_batch, s->d_a[0], s->d_status[0],
                                                          s->d_escale, K, s->d_res, s->d_rst);
    k_srv_done<<<1, 1, 0, ctx->stream>>>(s->dq, s->d_batch, ctx->d_err);
    if (cudaPeekAtLastError() != cudaSuccess) rc = GP_ERR_CUDA;
  }
  cudaGraph_t captured = NULL;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &captured);
  if (rc) return gp_fail(ctx, rc, "gp_serve_open: capturing the serving loop failed");
  if (e != cudaSuccess) return gp_cuda_fail(ctx, e, "gp_serve_open: cudaStreamEndCapture");
  GP_CUDA(ctx, cudaGraphInstantiate(&s->gexec, g, 0));
  GP_CUDA(ctx, cudaMemsetAsync(s->d_batch, 0, sizeof(gp_tc_batch), ctx->stream));
  GP_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GP_OK;
}

/* full-PCA worker: takes the front job when it fits the budget (or nothing else runs) */
struct worker_arg {
  gp_server *s;
  int index;
};

static void *pca_worker(void *arg)
{
  worker_arg *wa = (worker_arg *)arg;
  gp_server *s = wa->s;
  gp_ctx *ctx = s->wctx[(size_t)wa->index];
  delete wa;
  cudaSetDevice(ctx->device);
  pthread_mutex_lock(&s->mu);
  for (;;) {
    gp_req *j = NULL;
    /* a job starts only while the device-resident loop is stopped (the scheduler stops it
     * when jobs wait): the job's allocations synchronise the device */
    if (!s->pca_waiting.empty() && !s->loop_running) {
      gp_req *f = s->pca_waiting.front();
      if (s->pca_running == 0 || s->pca_used + f->footprint <= s->pca_budget) {
        j = f;
        s->pca_waiting.pop_front();
      }
    }
    if (!j) {
      if (s->stop && s->pca_waiting.empty()) break;
      pthread_cond_wait(&s->cv, &s->mu);
      continue;
    }
    s->pca_used += j->footprint;
    s->pca_running++;
    if (s->pca_running > s->pca_peak) s->pca_peak = s->pca_running;
    pthread_mutex_unlock(&s->mu);
    int rc = gp_smartpca_run(ctx, j->opts, j->panel, j->result);
    if (rc) snprintf(s->err, sizeof s->err, "PCA job %lld: %s", (long long)j->id, gp_last_error(ctx));
    gp_release(ctx);
    pthread_mutex_lock(&s->mu);
    s->pca_used -= j->footprint;
    s->pca_running--;
    s->pca_done++;
    j->error = rc;
    j->done = 1;
    pthread_cond_broadcast(&s->cv);
  }
  pthread_mutex_unlock(&s->mu);
  return NULL;
}

extern "C" int64_t gp_smartpca_footprint(int32_t nind, int64_t nsnp, int32_t precision,
                                         int32_t numeigs)
{
  const int64_t n = nind, m = nsnp, npad = (n + 127) / 128 * 128;
  const int64_t rec = m * ((n + 63) / 64 * 16);
  const int64_t gram = 8 * n * n;
  const int64_t k = numeigs > 0 ? numeigs : 1;
  /* the eigensolve's vectors and workspace, plus the tiled tridiagonalisation's lower-triangle
   * tiles (64 x 64 float-float pairs) and its parts (27 x 64 per index block of 64) */
  const int64_t nt = (n + 63) / 64;
  const int64_t eig = 8 * n * 64 + 48 * n * (k > 10 ? k : 10) + 8 * n * k +
                      8 * (nt * (nt + 1) / 2 * 64 * 64 + 27 * nt * 64 + 3 * nt) + 5 * nt * nt;
  int64_t work;
  if (precision == GP_PREC_FP64) {
    work = 8 * m * (k * (k + 1) / 2 + 1) + 8 * n * 256;
  } else {
    int64_t split = 4 * npad * m;
    if (split > (int64_t)24 << 30) split = (int64_t)24 << 30;
    const int64_t tc = n * (m / 4 + 16) + m * 1024 + n * 8 * 1024 + 8 * m * 256;
    work = split > tc ? split : tc;
  }
  return rec + gram + eig + work + 100 * m + ((int64_t)256 << 20);
}

/* ------------------------------------------------------------------------------------ */

extern "C" const char *gp_serve_last_error(const gp_server *srv) { return srv ? srv->err : ""; }

extern "C" void gp_serve_close(gp_server *s)
{
  if (!s) return;
  if (s->thread_started) {
    pthread_mutex_lock(&s->mu);
    s->stop = 1;
    s->paused = 0;
    pthread_cond_broadcast(&s->cv);
    pthread_mutex_unlock(&s->mu);
    pthread_join(s->thread, NULL);
  }
  if (!s->workers.empty()) {
    pthread_mutex_lock(&s->mu);
    s->stop = 1;
    pthread_cond_broadcast(&s->cv);
    pthread_mutex_unlock(&s->mu);
    for (pthread_t t : s->workers) pthread_join(t, NULL);
  }
  for (gp_ctx *w : s->wctx) gp_close(w);
  if (s->ctx) cudaSetDevice(s->ctx->device);
  if (s->ctx && s->loop_running && !s->thread_started) {
    /* opened the loop but not the thread: stop the loop here */
    __atomic_store_n(&s->hq->stop, 1, __ATOMIC_RELEASE);
    cudaStreamSynchronize(s->ctx->stream);
  }
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->graph) cudaGraphDestroy(s->graph);
  if (s->hq) cudaFreeHost(s->hq);
  if (s->h_res) cudaFreeHost(s->h_res);
  if (s->h_rst) cudaFreeHost(s->h_rst);
  void *dev[] = {s->d_E,     s->d_P,      s->d_fE,     s->d_mE,     s->d_otab,   s->d_rtab,
                 s->stor_co, s->stor_rr,  s->d_pool,   s->d_co[0],  s->d_co[1],  s->d_rr[0],
                 s->d_rr[1], s->d_a[0],   s->d_a[1],   s->d_b[0],   s->d_b[1],   s->d_work[0],
                 s->d_work[1], s->d_part[0], s->d_part[1], s->d_nobs[0], s->d_nobs[1],
                 s->d_status[0], s->d_status[1], s->d_batch, s->d_Z, s->d_escale};
  for (size_t i = 0; i < sizeof(dev) / sizeof(dev[0]); ++i)
    if (dev[i]) cudaFree(dev[i]);
  for (int i = 0; i < 2; ++i) {
    if (s->h_a[i]) cudaFreeHost(s->h_a[i]);
    if (s->h_status[i]) cudaFreeHost(s->h_status[i]);
    if (s->h_err[i]) cudaFreeHost(s->h_err[i]);
  }
  for (auto &kv : s->all) {
    if (kv.second->copied) cudaEventDestroy(kv.second->copied);
    delete kv.second;
  }
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->ctx) gp_close(s->ctx);
  pthread_mutex_destroy(&s->mu);
  pthread_cond_destroy(&s->cv);
  delete s;
}

extern "C" int gp_serve_open(gp_ctx *src, const gp_serve_opts *o, gp_server **out)
{
  if (!src || !o || !out) return GP_ERR_ARG;
  *out = NULL;
  if (!src->weights_valid)
    return gp_fail(src, GP_ERR_STATE, "gp_serve_open: the source handle has no SNP weights");
  const int32_t K = o->numeigs;
  if (K < 1 || K > src->nweights || K > 64)
    return gp_fail(src, GP_ERR_ARG, "gp_serve_open: numeigs %d out of range", K);
  if (src->nkept < 1) return gp_fail(src, GP_ERR_NODATA, "gp_serve_open: the panel has no SNP");
  gp_server *s = new gp_server();
  pthread_mutex_init(&s->mu, NULL);
  pthread_cond_init(&s->cv, NULL);
  s->K = K;
  s->npair = K * (K + 1) / 2;
  s->ldp = s->npair + 1;
  s->nk = src->nkept;
  s->row_bytes = (int64_t)((s->nk + 63) / 64) * 16;
  s->max_batch = o->max_batch > 0 ? o->max_batch : 4096;
  s->pool_cap = o->pool_samples > 0 ? o->pool_samples : 32768;
  if (s->pool_cap < s->max_batch) s->pool_cap = s->max_batch;
  s->fp64_serial = o->fp64_serial;
  s->host_loop = o->host_loop || o->fp64_serial;
  s->eigscale.assign((size_t)K, 1.0);
  if (o->eigscale)
    for (int32_t j = 0; j < K; ++j) s->eigscale[(size_t)j] = o->eigscale[j];
  int rc = gp_open(src->device, &s->ctx);
  if (rc) {
    snprintf(src->err, GP_ERRLEN, "gp_serve_open: %s", gp_last_error(NULL));
    delete s;
    return rc;
  }
  gp_ctx *ctx = s->ctx;
  const size_t nk = (size_t)s->nk;
  cudaError_t e = cudaSuccess;
#define SALLOC(p, bytes)                                   \
  if (e == cudaSuccess) e = cudaMalloc((void **)&(p), (bytes) < 256 ? 256 : (bytes))
  SALLOC(s->d_E, sizeof(double) * nk * K);
  SALLOC(s->d_P, sizeof(double) * nk * s->ldp);
  SALLOC(s->d_fE, sizeof(double) * nk * K);
  SALLOC(s->d_mE, sizeof(double) * nk * K);
  SALLOC(s->d_otab, sizeof(double) * nk * 4);
  SALLOC(s->d_rtab, sizeof(double) * nk * 4);
  SALLOC(s->d_pool, (size_t)s->pool_cap * s->row_bytes);
  for (int i = 0; i < 2; ++i) {
    SALLOC(s->d_co[i], sizeof(double) * (size_t)s->max_batch * s->ldp);
    SALLOC(s->d_rr[i], sizeof(double) * (size_t)s->max_batch * K);
    SALLOC(s->d_a[i], sizeof(double) * (size_t)s->max_batch * K);
    SALLOC(s->d_b[i], sizeof(double) * (size_t)s->max_batch * K);
    SALLOC(s->d_work[i], sizeof(double) * (size_t)s->max_batch * (K * K + 2 * K));
    SALLOC(s->d_nobs[i], sizeof(int32_t) * (size_t)s->max_batch);
    SALLOC(s->d_status[i], sizeof(int32_t) * (size_t)s->max_batch);
    if (s->fp64_serial) SALLOC(s->d_part[i], sizeof(double) * 16 * (size_t)s->max_batch * s->ldp);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&s->h_a[i], sizeof(double) * (size_t)s->max_batch * K, 0);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&s->h_status[i], sizeof(int32_t) * (size_t)s->max_batch, 0);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&s->h_err[i], sizeof(int) * 4, 0);
  }
  if (!s->fp64_serial) {
    size_t b1 = gp_tc_prepared_bytes(1, s->ldp, s->nk), b2 = gp_tc_prepared_bytes(2, K, s->nk);
    SALLOC(s->stor_co, b1);
    SALLOC(s->stor_rr, b2);
  }
  if (!s->host_loop) {
    /* the loop's queue and result rows in mapped pinned host memory, its batch state and the
     * products' slice-column buffer (normal-equation panel: the wider of the two) */
    const int64_t ncols4_pad = ((int64_t)4 * s->ldp + 127) / 128 * 128;
    SALLOC(s->d_batch, sizeof(gp_tc_batch));
    SALLOC(s->d_Z, sizeof(double) * (size_t)s->max_batch * ncols4_pad);
    SALLOC(s->d_escale, sizeof(double) * K);
    if (e == cudaSuccess)
      e = cudaHostAlloc((void **)&s->hq, sizeof(gp_srv_queue), cudaHostAllocMapped);
    if (e == cudaSuccess)
      e = cudaHostAlloc((void **)&s->h_res, sizeof(double) * (size_t)s->pool_cap * K,
                        cudaHostAllocMapped);
    if (e == cudaSuccess)
      e = cudaHostAlloc((void **)&s->h_rst, sizeof(int32_t) * (size_t)s->pool_cap,
                        cudaHostAllocMapped);
    if (e == cudaSuccess) {
      memset(s->hq, 0, sizeof(gp_srv_queue));
      e = cudaHostGetDevicePointer((void **)&s->dq, s->hq, 0);
    }
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_res, s->h_res, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_rst, s->h_rst, 0);
    if (e == cudaSuccess)
      e = cudaMemcpy(s->d_escale, s->eigscale.data(), sizeof(double) * K, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    /* panel SNP records, host side, for callers that build request rows */
    std::vector<int32_t> kept(nk), cols((size_t)src->ncols);
    cudaSetDevice(src->device);
    e = cudaMemcpy(kept.data(), src->d_kept, sizeof(int32_t) * nk, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(cols.data(), src->d_cols, sizeof(int32_t) * cols.size(), cudaMemcpyDeviceToHost);
    s->snp_index.resize(nk);
    for (size_t k = 0; k < nk && e == cudaSuccess; ++k) s->snp_index[k] = cols[(size_t)kept[k]];
  }
  if (e != cudaSuccess) {
    gp_fail(src, GP_ERR_NOMEM, "gp_serve_open: allocation failed: %s", cudaGetErrorString(e));
    gp_serve_close(s);
    return GP_ERR_NOMEM;
  }
  /* the panel: from the source handle's resident weights (its own stream, then wait) */
  GP_CUDA(src, cudaSetDevice(src->device));
  if (s->nk > 0) {
    int blocks = (int)((nk + 127) / 128);
    if (blocks > src->num_sms * 8) blocks = src->num_sms * 8;
    k_serve_panel<<<blocks, 128, 0, src->stream>>>(src->d_ffvecs, src->d_fxscal, src->d_kept,
                                                   src->d_xfancy, src->d_xmean, s->nk, src->ncols,
                                                   K, s->d_E, s->d_P, s->ldp, s->d_fE, s->d_mE,
                                                   s->d_otab, s->d_rtab);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(src->stream);
    if (e != cudaSuccess) {
      gp_cuda_fail(src, e, "k_serve_panel");
      gp_serve_close(s);
      return GP_ERR_CUDA;
    }
  }
  if (!s->fp64_serial && s->nk > 0) {
    gp_tc_panel pc = {s->d_P, s->ldp, 1.0, 0};
    rc = gp_tc_prepare(ctx, 1, &pc, s->ldp, s->nk, s->stor_co, &s->Pco);
    gp_tc_panel pr[2] = {{s->d_fE, K, 1.0, 1}, {s->d_mE, K, -1.0, 0}};
    if (!rc) rc = gp_tc_prepare(ctx, 2, pr, K, s->nk, s->stor_rr, &s->Prr);
    /* the products' slice-column buffer, sized once for the largest batch */
    void *z;
    if (!rc) rc = gp_scratch5(ctx, (size_t)s->max_batch * s->Pco.ncols4_pad * 8 + 256, &z);
    if (!rc) {
      e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = gp_cuda_fail(ctx, e, "gp_serve_open prepare");
    }
    if (rc) {
      snprintf(src->err, GP_ERRLEN, "gp_serve_open: %s", gp_last_error(ctx));
      gp_serve_close(s);
      return rc;
    }
  }
  if (!s->host_loop && s->nk > 0) {
    rc = build_loop(s);
    if (rc) {
      snprintf(src->err, GP_ERRLEN, "%s", gp_last_error(ctx));
      gp_serve_close(s);
      return rc;
    }
  }
  /* full-PCA workers, each with its own handle (stream, solver) */
  s->pca_budget = o->pca_budget_bytes > 0 ? o->pca_budget_bytes : ((int64_t)64 << 30);
  const int nw = o->pca_workers > 0 ? (o->pca_workers > 8 ? 8 : o->pca_workers) : 1;
  for (int i = 0; i < nw; ++i) {
    gp_ctx *w = NULL;
    if (gp_open(src->device, &w) != GP_OK) break;
    s->wctx.push_back(w);
    worker_arg *wa = new worker_arg{s, i};
    pthread_t t;
    if (pthread_create(&t, NULL, pca_worker, wa) != 0) {
      delete wa;
      break;
    }
    s->workers.push_back(t);
  }
  if (s->workers.empty()) {
    gp_fail(src, GP_ERR_STATE, "gp_serve_open: could not start a PCA worker");
    gp_serve_close(s);
    return GP_ERR_STATE;
  }
  if (pthread_create(&s->thread, NULL, scheduler, s) != 0) {
    gp_fail(src, GP_ERR_STATE, "gp_serve_open: could not start the scheduler thread");
    gp_serve_close(s);
    return GP_ERR_STATE;
  }
  s->thread_started = 1;
  if (s->gexec) {
    /* the loop: launched once the workers' handles exist (their creation may allocate) */
    pthread_mutex_lock(&s->mu);
    if (!s->loop_running) start_loop(s);
    pthread_mutex_unlock(&s->mu);
  }
  *out = s;
  return GP_OK;
}

extern "C" int gp_serve_layout(const gp_server *s, int64_t *nsnp, int64_t *row_bytes)
{
  if (!s) return GP_ERR_ARG;
  if (nsnp) *nsnp = s->nk;
  if (row_bytes) *row_bytes = s->row_bytes;
  return GP_OK;
}

extern "C" int gp_serve_panel_snps(const gp_server *s, int32_t *snp_index)
{
  if (!s || !snp_index) return GP_ERR_ARG;
  memcpy(snp_index, s->snp_index.data(), sizeof(int32_t) * s->snp_index.size());
  return GP_OK;
}

extern "C" int gp_serve_submit(gp_server *s, const uint8_t *codes, int32_t nsamp, double *coords,
                               int32_t *status, int64_t *ticket)
{
  if (!s || !codes || !coords || !status || !ticket || nsamp < 1) return GP_ERR_ARG;
  if (nsamp > s->max_batch || nsamp > s->pool_cap)
    return srv_fail(s, GP_ERR_FULL, "request larger than the batch or the device pool");
  gp_req *r = new gp_req();
  r->nsamp = nsamp;
  r->codes = codes;
  r->coords = coords;
  r->status = status;
  if (cudaEventCreateWithFlags(&r->copied, cudaEventDisableTiming) != cudaSuccess) {
    delete r;
    return srv_fail(s, GP_ERR_CUDA, "cudaEventCreate failed");
  }
  pthread_mutex_lock(&s->mu);
  r->id = s->next_id++;
  s->all[r->id] = r;
  s->waiting.push_back(r);
  admit_waiting(s);
  pthread_cond_broadcast(&s->cv);
  pthread_mutex_unlock(&s->mu);
  *ticket = r->id;
  return GP_OK;
}

extern "C" int gp_serve_submit_pca(gp_server *s, const gp_panel *panel,
                                   const gp_smartpca_opts *opts, gp_run_result *result,
                                   int64_t *ticket)
{
  if (!s || !panel || !opts || !result || !ticket || !panel->records) return GP_ERR_ARG;
  gp_req *r = new gp_req();
  r->kind = 1;
  r->panel = panel;
  r->opts = opts;
  r->result = result;
  r->footprint = gp_smartpca_footprint(panel->nind, panel->nsnp, opts->precision, opts->numeigs);
  pthread_mutex_lock(&s->mu);
  r->id = s->next_id++;
  s->all[r->id] = r;
  s->pca_waiting.push_back(r);
  pthread_cond_broadcast(&s->cv);
  pthread_mutex_unlock(&s->mu);
  *ticket = r->id;
  return GP_OK;
}

extern "C" int gp_serve_pca_stats(const gp_server *s, int64_t *jobs_done, int32_t *peak_running,
                                  int64_t *bytes_in_use)
{
  if (!s) return GP_ERR_ARG;
  gp_server *m = (gp_server *)s;
  pthread_mutex_lock(&m->mu);
  if (jobs_done) *jobs_done = s->pca_done;
  if (peak_running) *peak_running = s->pca_peak;
  if (bytes_in_use) *bytes_in_use = s->pca_used;
  pthread_mutex_unlock(&m->mu);
  return GP_OK;
}

extern "C" int gp_serve_test(gp_server *s, int64_t ticket)
{
  if (!s) return GP_ERR_ARG;
  pthread_mutex_lock(&s->mu);
  auto it = s->all.find(ticket);
  int rc;
  if (it == s->all.end()) {
    rc = GP_ERR_ARG;
  } else if (!it->second->done) {
    rc = 0;
  } else {
    rc = it->second->error ? it->second->error : 1;
    delete it->second;
    s->all.erase(it);
  }
  pthread_mutex_unlock(&s->mu);
  return rc;
}

extern "C" int gp_serve_wait(gp_server *s, int64_t ticket, double timeout_s)
{
  if (!s) return GP_ERR_ARG;
  struct timespec dl;
  clock_gettime(CLOCK_REALTIME, &dl);
  double t = (double)dl.tv_sec + 1e-9 * dl.tv_nsec + (timeout_s > 0 ? timeout_s : 0.0);
  dl.tv_sec = (time_t)t;
  dl.tv_nsec = (long)((t - (double)dl.tv_sec) * 1e9);
  pthread_mutex_lock(&s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) {
    pthread_mutex_unlock(&s->mu);
    return srv_fail(s, GP_ERR_ARG, "unknown ticket");
  }
  gp_req *r = it->second;
  int rc = GP_OK;
  while (!r->done) {
    int w = pthread_cond_timedwait(&s->cv, &s->mu, &dl);
    if (w == ETIMEDOUT && !r->done) {
      rc = GP_ERR_TIMEOUT;
      snprintf(s->err, sizeof s->err, "request %lld still pending after %.3f s",
               (long long)ticket, timeout_s);
      break;
    }
  }
  if (r->done) {
    if (r->error) rc = r->error;
    s->all.erase(ticket); /* by key: inserts meanwhile may have rehashed the map */
    delete r;
  }
  pthread_mutex_unlock(&s->mu);
  return rc;
}

extern "C" int gp_serve_pause(gp_server *s, int32_t paused)
{
  if (!s) return GP_ERR_ARG;
  pthread_mutex_lock(&s->mu);
  s->paused = paused ? 1 : 0;
  pthread_cond_broadcast(&s->cv);
  /* a pause returns once the device-resident loop has stopped, so that the caller may then
   * make calls that synchronise the device */
  while (s->paused && s->loop_running && s->thread_started)
    pthread_cond_wait(&s->cv, &s->mu);
  pthread_mutex_unlock(&s->mu);
  return GP_OK;
}

extern "C" int gp_serve_loop_stats(const gp_server *s, int32_t *device_loop, int64_t *launches,
                                   int64_t *batches, int64_t *idle_polls)
{
  if (!s) return GP_ERR_ARG;
  gp_server *m = (gp_server *)s;
  pthread_mutex_lock(&m->mu);
  if (device_loop) *device_loop = s->loop_running;
  if (launches) *launches = s->loop_launches;
  if (batches) *batches = s->hq ? *(volatile int64_t *)&s->hq->batches : s->n_batches;
  if (idle_polls) *idle_polls = s->hq ? *(volatile int64_t *)&s->hq->idle_polls : 0;
  pthread_mutex_unlock(&m->mu);
  return GP_OK;
}

extern "C" int gp_serve_stats(const gp_server *s, int64_t *batches, int64_t *samples,
                              int64_t *requests)
{
  if (!s) return GP_ERR_ARG;
  gp_server *m = (gp_server *)s;
  pthread_mutex_lock(&m->mu);
  if (batches) *batches = s->n_batches;
  if (samples) *samples = s->n_samples;
  if (requests) *requests = s->n_requests;
  pthread_mutex_unlock(&m->mu);
  return GP_OK;
}
