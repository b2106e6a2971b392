/*
 * gp_gram_fp64_noalloc: the FP64 Gram of a small genotype panel without any device memory
 * allocation, for callers that cannot allocate.
 *
 * Who needs it: a host application whose memory manager has reserved the whole device for
 * its own pool (common in long-running serving processes, where a cudaMalloc would fail or
 * would fragment the pool), or a latency-critical loop that must not call cudaMalloc /
 * cudaFree because they can synchronise the device.  Such a caller owns every buffer it
 * passes in; this entry point only needs scratch for its split-K partial sums, and takes it
 * from a fixed array compiled into the library.
 *
 * The scratch is a file-scope __device__ array of GP_NOALLOC_SCRATCH_DOUBLES doubles
 * (16 MiB).  Every GPU that loads the library holds it until the process exits.  Host code
 * cannot use the array's name as a device address, so the first call on each device (with
 * that device current) looks the address up with cudaGetSymbolAddress and caches it; make
 * that first call before any stream capture begins.  With CUDA's lazy module loading (the
 * default since CUDA 12.2) the array itself is only allocated when this code is first used on
 * a device, i.e. by that first call: a caller whose pool reserves the whole device must make
 * the first call before the pool takes the memory.  The cached address is not refreshed after
 * a cudaDeviceReset of that device (which frees the array): after a reset the entry point must
 * not be used again in that process.  All calls share the one array and it keeps the last
 * call's contents: each call overwrites every scratch entry it later reads, and calls whose
 * work overlaps on the GPU (different streams, or different host threads on one stream
 * without ordering) race on it.  The host side is thread-safe: the address lookup happens
 * once per device under a lock, and the failure text is kept per host thread.
 */
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "gp_internal.h"

#define GP_NOALLOC_SCRATCH_DOUBLES (2 * 1024 * 1024) /* 16 MiB */
#define GP_NOALLOC_MAX_NIND 1024                      /* largest panel accepted */
#define NT 64                                         /* tile edge */
#define NK 16                                         /* SNPs per k-step */
#define GP_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[GP_NOALLOC_SCRATCH_DOUBLES];

static std::atomic<double *> g_noalloc_addr[GP_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_lookup;

static thread_local char g_noalloc_err[256];

/* partial[s][i][j] (j <= i) = sum over SNPs of split s of v_i v_j for one 64x64 tile */
__global__ void __launch_bounds__(256)
k_gram_f64_noalloc(const uint8_t *__restrict__ rec, int64_t rlen, int32_t n, int32_t nsnp,
                   const double *__restrict__ vtab, int32_t kper, double *part)
{
  __shared__ double As[NK][NT + 1];
  __shared__ double Bs[NK][NT + 1];
  int32_t t = (int32_t)blockIdx.x;
  int32_t bi = (int32_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((bi + 1) * (bi + 2) / 2 <= t) ++bi;
  while (bi * (bi + 1) / 2 > t) --bi;
  int32_t bj = t - bi * (bi + 1) / 2;
  const int32_t i0 = bi * NT, j0 = bj * NT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int lk = tid & 15, lr = tid >> 4;
  const int32_t k0 = (int32_t)blockIdx.y * kper;
  const int32_t k1 = k0 + kper < nsnp ? k0 + kper : nsnp;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int32_t ks = k0; ks < k1; ks += NK) {
    int32_t s = ks + lk;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int32_t ri = i0 + lr + 16 * q, rj = j0 + lr + 16 * q;
      double va = 0.0, vb = 0.0;
      if (s < k1) {
        const uint8_t *r = rec + (int64_t)s * rlen;
        if (ri < n) va = vtab[4 * s + ((r[ri >> 2] >> ((3 - (ri & 3)) * 2)) & 3)];
        if (rj < n) vb = vtab[4 * s + ((r[rj >> 2] >> ((3 - (rj & 3)) * 2)) & 3)];
      }
      As[lk][lr + 16 * q] = va;
      Bs[lk][lr + 16 * q] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[k][ty + 16 * q];
        b[q] = Bs[k][tx + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
  double *o = part + (int64_t)blockIdx.y * n * n;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    int32_t i = i0 + ty + 16 * p;
    if (i >= n) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int32_t j = j0 + tx + 16 * q;
      if (j < n && j <= i) o[(int64_t)i * n + j] = acc[p][q];
    }
  }
}

/* xtx = sum of the partials in split order, both triangles */
__global__ void k_noalloc_reduce(double *xtx, const double *part, int32_t nsplit, int32_t n)
{
  int64_t total = (int64_t)n * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = idx / n, j = idx - i * n;
    int64_t lo = i >= j ? idx : j * n + i;
    double s = 0.0;
    for (int32_t t = 0; t < nsplit; ++t) s += part[t * total + lo];
    xtx[idx] = s;
  }
}

static int noalloc_fail(int code, const char *msg)
{
  snprintf(g_noalloc_err, sizeof g_noalloc_err, "%s", msg);
  return code;
}

extern "C" const char *gp_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" int gp_gram_fp64_noalloc(const uint8_t *d_records, int64_t record_bytes,
                                    int32_t nind, int32_t nsnp, const double *d_vtab,
                                    double *d_xtx, void *stream)
{
  if (!d_records || !d_vtab || !d_xtx || nind < 1 || nsnp < 1 ||
      record_bytes < ((int64_t)nind + 3) / 4)
    return noalloc_fail(GP_ERR_ARG, "gp_gram_fp64_noalloc: bad arguments");
  if (nind > GP_NOALLOC_MAX_NIND)
    return noalloc_fail(GP_ERR_ARG,
                        "gp_gram_fp64_noalloc: nind exceeds the fixed scratch limit of 1024 "
                        "samples (use gp_xtx)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= GP_NOALLOC_MAX_DEVICES)
    return noalloc_fail(GP_ERR_CUDA, "gp_gram_fp64_noalloc: no usable current device");
  double *part = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (!part) {
    /* once per device, with that device current: the array's device address */
    std::lock_guard<std::mutex> lock(g_noalloc_lookup);
    part = g_noalloc_addr[dev].load(std::memory_order_acquire);
    if (!part) {
      e = cudaGetSymbolAddress((void **)&part, g_noalloc_scratch);
      if (e != cudaSuccess || !part)
        return noalloc_fail(GP_ERR_CUDA, "gp_gram_fp64_noalloc: cudaGetSymbolAddress failed");
      g_noalloc_addr[dev].store(part, std::memory_order_release);
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nn = (int64_t)nind * nind;
  const int32_t nt = (nind + NT - 1) / NT, ntiles = nt * (nt + 1) / 2;
  int32_t nsplit = (int32_t)(GP_NOALLOC_SCRATCH_DOUBLES / nn);
  int32_t want = (256 + ntiles - 1) / ntiles; /* enough blocks to fill the GPU */
  if (nsplit > want) nsplit = want;
  if (nsplit > (nsnp + NK - 1) / NK) nsplit = (nsnp + NK - 1) / NK;
  if (nsplit < 1) nsplit = 1;
  int32_t kper = (nsnp + nsplit - 1) / nsplit;
  kper = (kper + NK - 1) / NK * NK;
  nsplit = (nsnp + kper - 1) / kper;
  /* no clearing needed: every split has SNPs (nsplit = ceil(nsnp / kper)) and its tiles write
   * every lower-triangle entry i < nind, j <= i of its slice, the only entries the reduction
   * reads */
  dim3 grid((unsigned)ntiles, (unsigned)nsplit);
  k_gram_f64_noalloc<<<grid, 256, 0, st>>>(d_records, record_bytes, nind, nsnp, d_vtab, kper, part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(GP_ERR_CUDA, cudaGetErrorString(e));
  int blocks = (int)((nn + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  k_noalloc_reduce<<<blocks, 256, 0, st>>>(d_xtx, part, nsplit, nind);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(GP_ERR_CUDA, cudaGetErrorString(e));
  return GP_OK;
}
