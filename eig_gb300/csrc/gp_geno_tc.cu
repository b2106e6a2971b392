/*
 * Exact genotype x FP64-panel products on the tensor cores.
 *
 *   Y[r][c] = sum_k A_r(k) P[k][c]
 *
 * A_r(k) is a small integer decoded from a 2-bit genotype code through a 4-entry table
 * (observed mask {1,1,1,0} or allele count {0,1,2,0}); P is an FP64 panel.  Each column of
 * P is scaled by a power of two 2^e_c >= max|P[.][c]| and cut into 4 fixed-point slices,
 * x = P/2^e_c = sum_t q_t 1024^-(t+1) with |q_0| <= 1024 and |q_t| <= 512 (t > 0): integers
 * that fp16 holds exactly.  A tensor-core MMA of {0,1,2} by such integers over at most 8,192
 * k values sums to an integer below 2^24, which FP32 holds exactly, so the FP32 accumulation
 * of the MMA loses nothing; chunk sums are added in int32 registers and flushed with FP64
 * atomics of exact integers (order-independent, hence deterministic).  The only error left
 * is the slicing, about 2^-41 of the column maximum.
 *
 * This is how the masked per-sample normal equations of lsqproject (regressit
 * src/regsubs.c:19-26, lsqproj src/eigensrc/smartpca.c:4690-4712), the sample scores fxvecs
 * and the SNP weights ffvecs (smartpca.c:1485-1525) reach FP64 accuracy at tensor-core
 * speed.  Both orientations use the same kernel; only the operand layout differs:
 *   sum over SNPs     rows = samples, k = kept SNPs (codes in sample-major order)
 *   sum over samples  rows = kept SNPs, k = samples (codes in SNP-major order)
 *
 * Kernel structure (grid-stride over work items = row tile x column tile x k-split, the row
 * tile fastest, so that the CTAs running at one time share the B tile and k range they
 * stream and B is read from DRAM about once per wave instead of once per row tile):
 *   warp 0      TMA of the B tile (128 slice-columns x 64 k, fp16, 128-byte swizzle);
 *   warp 1      one thread issues 4 tcgen05.mma (128x128x16, f16 -> f32) per k-block into
 *               TMEM buffer (chunk & 1);
 *   warps 2-9   decode the A tile, two threads per row: each reads 8 bytes of codes (32 k;
 *               the next eight k-blocks' loads in flight) and writes 32 fp16 values into
 *               shared memory in the same swizzled layout, each code turned into its fp16
 *               value by a byte permute of the 4-entry table held in two registers; then
 *               fence.proxy.async + mbarrier arrive (the decode bounds the kernel: four
 *               decoder warps, one thread per row, left the tensor pipe ~20% busy);
 *   warps 10-17 epilogue: per chunk tcgen05.ld the exact FP32 sums, add into int32
 *               registers (64 columns per thread), flush with FP64 atomics per work item.
 */
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <math.h>

#include "gp_geno_tc.h"
#include "gp_tc.cuh"

#define XT 128              /* rows / slice-columns per tile */
#define XK 64               /* k per k-block */
#define XSTAGES 4
#define XA_BYTES (XT * XK * 2)
#define XB_BYTES (XT * XK * 2)
#define XSTAGE_BYTES (XA_BYTES + XB_BYTES)
#define X_THREADS 576       /* 18 warps */
#define X_DEC_WARPS 8       /* decoder warps: two threads per row of the A tile */
#define X_SMEM (XSTAGES * XSTAGE_BYTES + 1024 + 256)
#define X_CHUNK_KB 128      /* 8,192 k per exact FP32 chunk */
#define XPF 8               /* k-blocks of codes a decoder thread loads ahead */

#define XERR_FULL 11
#define XERR_EMPTY 12
#define XERR_ACCF 13
#define XERR_ACCE 14

/* fp16 bit patterns of the 4-entry decode tables */
#define H0 0x0000ull
#define H1 0x3C00ull
#define H2 0x4000ull
static const uint64_t LUT_MASK = H1 | (H1 << 16) | (H1 << 32);      /* {1,1,1,0} */
static const uint64_t LUT_COUNT = H0 | (H1 << 16) | (H2 << 32);     /* {0,1,2,0} */

__device__ __forceinline__ void fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

/*
 * codes: rows of ldc bytes (2-bit codes, MSB first, 3 = missing -> 0); output row r reads
 * code row row_map[r] (r itself when row_map is NULL); its k-block kb is the 16 bytes at
 * (kb % kb_period)*16, decoded with lut_lo for kb < kb_switch and lut_hi otherwise (the
 * concatenated-k form [G | O]).
 * zout: [nrows][ldz] FP64, receives atomically the exact integer sums per slice-column.
 */
__global__ void __launch_bounds__(X_THREADS, 1)
k_geno_panel_tc(const __grid_constant__ CUtensorMap tm_b, const uint8_t *__restrict__ codes,
                int64_t ldc, const int32_t *__restrict__ row_map, int32_t nrows, int32_t ncols4,
                int32_t nkb, int32_t kb_period,
                int32_t kb_switch, uint64_t lut_lo, uint64_t lut_hi, int32_t ksplit,
                double *zout, int64_t ldz, int *err, const gp_tc_batch *db)
{
  if (db) {
    /* a device-resident loop's batch: rows and their count are read at run time, and the
     * k split is chosen as gp_tc_apply chooses it for that count */
    codes = db->codes;
    nrows = db->nrows;
    const int32_t tiles = ((nrows + XT - 1) / XT) * ((ncols4 + XT - 1) / XT);
    ksplit = 1;
    while (tiles * ksplit < 2 * (int32_t)gridDim.x && ksplit * 4 <= nkb) ksplit *= 2;
    while ((int64_t)((nkb + ksplit - 1) / ksplit) * XK > (1 << 19)) ksplit *= 2;
  }
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + XSTAGES * XSTAGE_BYTES);
  uint64_t *full = bars, *empty = bars + XSTAGES, *accf = bars + 2 * XSTAGES,
           *acce = bars + 2 * XSTAGES + 2, *drain = bars + 2 * XSTAGES + 4;
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * XSTAGES + 5);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  const int32_t nrt = (nrows + XT - 1) / XT, nct = (ncols4 + XT - 1) / XT;
  const int32_t nitems = nrt * nct * ksplit;
  const int32_t kb_per = (nkb + ksplit - 1) / ksplit;

  if (threadIdx.x == 0) {
    for (int s = 0; s < XSTAGES; ++s) {
      mbar_init(&full[s], 1 + 32 * X_DEC_WARPS);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 8);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 0 && lane == 0) tma_prefetch_desc(&tm_b);
  if (warp == 1) tmem_alloc(tmem_slot, 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    /* ---------------- B producer (TMA) ---------------- */
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int32_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
        int32_t ks = (w / nrt) % ksplit, ct = w / (nrt * ksplit);
        int32_t kb0 = ks * kb_per, kb1 = kb0 + kb_per < nkb ? kb0 + kb_per : nkb;
        for (int32_t kb = kb0; kb < kb1; ++kb, ++it) {
          uint32_t s = it % XSTAGES, ph = (it / XSTAGES) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag, err, XERR_EMPTY)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&full[s], XB_BYTES);
          tma_load_2d(smem + s * XSTAGE_BYTES + XA_BYTES, &tm_b, &full[s], kb * XK, ct * XT);
        }
      }
      if (*abort_flag) {
        uint32_t last = it < XSTAGES ? it : XSTAGES;
        for (uint32_t j = it - last; j < it; ++j) {
          uint64_t t0 = globaltimer_ns();
          while (!mbar_try_wait(&full[j % XSTAGES], (j / XSTAGES) & 1u) &&
                 globaltimer_ns() - t0 < GP_WAIT_NS) {
          }
        }
      }
    }
  } else if (warp == 1) {
    /* ---------------- MMA issuer ---------------- */
    if (lane == 0) {
      const uint32_t idesc = idesc_f16_f32(XT, XT);
      uint32_t it = 0, chunk = 0;
      bool ok = true;
      for (int32_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
        int32_t ks = (w / nrt) % ksplit;
        int32_t kb0 = ks * kb_per, kb1 = kb0 + kb_per < nkb ? kb0 + kb_per : nkb;
        for (int32_t c0 = kb0; c0 < kb1 && ok; c0 += X_CHUNK_KB, ++chunk) {
          int32_t c1 = c0 + X_CHUNK_KB < kb1 ? c0 + X_CHUNK_KB : kb1;
          uint32_t buf = chunk & 1u, use = chunk >> 1;
          if (!mbar_wait(&acce[buf], (use & 1u) ^ 1u, abort_flag, err, XERR_ACCE)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + buf * XT;
          for (int32_t kb = c0; kb < c1; ++kb, ++it) {
            uint32_t s = it % XSTAGES, ph = (it / XSTAGES) & 1u;
            if (!mbar_wait(&full[s], ph, abort_flag, err, XERR_FULL)) {
              ok = false;
              break;
            }
            tc_fence_after();
            uint32_t base = smem_u32(smem + s * XSTAGE_BYTES);
            uint64_t ad = sdesc_k128(base), bd = sdesc_k128(base + XA_BYTES);
#pragma unroll
            for (int k = 0; k < XK / 16; ++k)
              umma_bf16(d, ad + (uint64_t)(2 * k), bd + (uint64_t)(2 * k), idesc,
                        (kb > c0 || k > 0) ? 1u : 0u);
            umma_commit(&empty[s]);
          }
          if (!ok) break;
          umma_commit(&accf[buf]);
        }
      }
    }
  } else if (warp < 2 + X_DEC_WARPS) {
    /* ---------------- A decoders: two threads per row of the tile ---------------- */
    const int dt = (warp - 2) * 32 + lane, r = dt >> 1, hb = dt & 1;
    /* the 4-entry fp16 tables as byte tables for prmt: code c is bytes 2c, 2c+1 */
    const uint32_t tlo0 = (uint32_t)lut_lo, tlo1 = (uint32_t)(lut_lo >> 32);
    const uint32_t thi0 = (uint32_t)lut_hi, thi1 = (uint32_t)(lut_hi >> 32);
    uint32_t it = 0;
    bool ok = true;
    for (int32_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
      int32_t ks = (w / nrt) % ksplit, rt = w % nrt;
      int32_t kb0 = ks * kb_per, kb1 = kb0 + kb_per < nkb ? kb0 + kb_per : nkb;
      const int32_t grow = rt * XT + r;
      const int64_t crow_idx = grow < nrows ? (row_map ? (int64_t)row_map[grow] : (int64_t)grow) : 0;
      const uint8_t *crow = codes + crow_idx * ldc + 8 * hb;
      /* this thread's half (8 bytes, 32 codes) of the row's codes of the next XPF k-blocks are
       * loaded ahead of the stage waits (the k-block index wraps at kb_period, so loads past
       * kb1 stay inside the row) */
      const bool live = grow < nrows;
      auto ld_codes = [&](int32_t kbx) {
        return live ? __ldg((const uint2 *)(crow + (int64_t)(kbx % kb_period) * 16))
                    : make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
      };
      uint2 pf[XPF];
#pragma unroll
      for (int u = 0; u < XPF; ++u) pf[u] = ld_codes(kb0 + u);
      for (int32_t kbb = kb0; kbb < kb1 && ok; kbb += XPF) {
#pragma unroll
        for (int u = 0; u < XPF; ++u) {
          const int32_t kb = kbb + u;
          if (kb >= kb1) break;
          const uint2 raw = pf[u];
          pf[u] = ld_codes(kb + XPF);
          uint32_t s = it % XSTAGES, ph = (it / XSTAGES) & 1u;
          ++it;
          bool got = mbar_wait(&empty[s], ph ^ 1u, abort_flag, err, XERR_EMPTY);
          if (!got) {
            ok = false;
            break;
          }
          const bool hi_tab = kb >= kb_switch;
          const uint32_t t0 = hi_tab ? thi0 : tlo0, t1 = hi_tab ? thi1 : tlo1;
          uint8_t *row_base = smem + s * XSTAGE_BYTES + r * 128;
          const uint32_t words[2] = {raw.x, raw.y};
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            /* codes 8j..8j+7 (j = 4 hb + jj): bytes 2j, 2j+1 of the row's 16 (little-endian
             * words); a byte holds four codes, MSB first, and each code c selects bytes 2c,
             * 2c+1 of the table */
            const int j = 4 * hb + jj;
            const uint32_t wv = words[jj >> 1] >> ((jj & 1) * 16);
            uint32_t outv[4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint32_t b = (wv >> (8 * h)) & 0xFFu;
              const uint32_t sel01 = ((b >> 6) & 3u) * 0x22u + ((b >> 4) & 3u) * 0x2200u + 0x1010u;
              const uint32_t sel23 = ((b >> 2) & 3u) * 0x22u + (b & 3u) * 0x2200u + 0x1010u;
              outv[2 * h] = __byte_perm(t0, t1, sel01);
              outv[2 * h + 1] = __byte_perm(t0, t1, sel23);
            }
            *(uint4 *)(row_base + ((j ^ (r & 7)) * 16)) =
                make_uint4(outv[0], outv[1], outv[2], outv[3]);
          }
          fence_proxy_async_smem();
          mbar_arrive(&full[s]);
        }
      }
    }
  } else {
    /* ---------------- epilogue: warps 2 + X_DEC_WARPS .. (8 warps) ---------------- */
    const int q = warp & 3, half = (warp - 2 - X_DEC_WARPS) >> 2;
    const int row = q * 32 + lane;
    const int col0 = half * 64;
    const uint32_t t_acc = tmem + ((uint32_t)(q * 32) << 16);
    uint32_t chunk = 0;
    bool ok = true;
    for (int32_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
      int32_t ks = (w / nrt) % ksplit, ct = w / (nrt * ksplit), rt = w % nrt;
      int32_t kb0 = ks * kb_per, kb1 = kb0 + kb_per < nkb ? kb0 + kb_per : nkb;
      int32_t acc[64];
#pragma unroll
      for (int u = 0; u < 64; ++u) acc[u] = 0;
      for (int32_t c0 = kb0; c0 < kb1; c0 += X_CHUNK_KB, ++chunk) {
        uint32_t buf = chunk & 1u, use = chunk >> 1;
        bool got = mbar_wait(&accf[buf], use & 1u, abort_flag, err, XERR_ACCF);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          uint32_t f[16];
          tmem_ld16(t_acc + buf * XT + col0 + 16 * g, f);
          tmem_wait_ld();
#pragma unroll
          for (int v = 0; v < 16; ++v) acc[16 * g + v] += __float2int_rn(__uint_as_float(f[v]));
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[buf]);
      }
      if (!ok) break;
      const int32_t grow = rt * XT + row;
      if (grow < nrows) {
        double *zr = zout + (int64_t)grow * ldz;
#pragma unroll
        for (int u = 0; u < 64; ++u) {
          int32_t gc = ct * XT + col0 + u;
          if (gc < ncols4 && acc[u] != 0) atomicAdd(zr + gc, (double)acc[u]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    if (*abort_flag && lane == 0) {
      umma_commit(drain);
      uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(drain, 0) && globaltimer_ns() - t0 < GP_WAIT_NS) {
      }
    }
    __syncwarp();
    tmem_dealloc(tmem, 256);
  }
}

/* ------------------------------------------------------------------------------------ */
/* operand preparation                                                                    */

/*
 * sum over SNPs: codes[r][k] = code of sample samp[r] at kept SNP k (record snprec[k]);
 * row stride ldc bytes; pad k (>= nk) and pad rows are 3.  A transpose through shared
 * memory: CTA (kt, rt) covers 128 kept SNPs x 128 rows; when the rows' samples span at most
 * CB_SPAN record bytes, the 128 records' byte ranges are read once (coalesced), and two
 * threads build each row's 32 output bytes; wider spans read per thread.
 */
#define CB_SNP 128
#define CB_ROWS 128
#define CB_SPAN 64
#define CB_PITCH_W (CB_SPAN / 4 + 1)
__global__ void __launch_bounds__(256)
k_codes_by_sample(const uint8_t *__restrict__ geno, int64_t rlen, const int32_t *__restrict__ samp,
                  int32_t nsamp, int32_t nrows_pad, const int32_t *__restrict__ snprec, int32_t nk,
                  int64_t ldc, uint8_t *codes)
{
  __shared__ uint32_t srec[CB_SNP][CB_PITCH_W];
  __shared__ int64_t soff[CB_SNP];
  const int tid = threadIdx.x;
  const int32_t r0 = blockIdx.y * CB_ROWS;
  int32_t base = 0, span = 0;
  if (r0 < nsamp) {
    const int32_t rl = (r0 + CB_ROWS < nsamp ? r0 + CB_ROWS : nsamp) - 1;
    base = (samp[r0] >> 2) & ~15;
    span = (samp[rl] >> 2) - base + 1;
  }
  const bool fast = span <= CB_SPAN;
  const int rl = tid >> 1, half = tid & 1;
  const int32_t r = r0 + rl;
  const int32_t sidx = r < nsamp ? samp[r] : 0;
  /* the CTA walks the SNP tiles of its row block (grid-stride over x) */
  const int32_t nkt = (int32_t)((ldc * 4 + CB_SNP - 1) / CB_SNP);
  for (int32_t kt = blockIdx.x; kt < nkt; kt += gridDim.x) {
    const int32_t k0 = kt * CB_SNP;
    if (tid < CB_SNP) soff[tid] = (k0 + tid < nk) ? (int64_t)snprec[k0 + tid] * rlen : -1;
    __syncthreads();
    if (fast && span > 0) {
      const int nvec = (span + 15) >> 4;
      for (int i = tid; i < CB_SNP * nvec; i += blockDim.x) {
        const int u = i / nvec, v = i - u * nvec;
        uint4 val = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
        if (soff[u] >= 0) val = __ldg((const uint4 *)(geno + soff[u] + base + 16 * v));
        srec[u][4 * v] = val.x;
        srec[u][4 * v + 1] = val.y;
        srec[u][4 * v + 2] = val.z;
        srec[u][4 * v + 3] = val.w;
      }
    }
    __syncthreads();
    if (r < nrows_pad && (int64_t)k0 + 64 * half < ldc * 4) {
      uint32_t out[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
      if (r < nsamp) {
        const int32_t bb = (sidx >> 2) - base, sh = (3 - (sidx & 3)) * 2;
#pragma unroll 8
        for (int j = 0; j < 64; ++j) {
          const int u = 64 * half + j;
          uint32_t byte = 0xFFu;
          if (soff[u] >= 0)
            byte = fast ? (srec[u][bb >> 2] >> ((bb & 3) * 8)) & 0xFFu
                        : __ldg(geno + soff[u] + (sidx >> 2));
          const uint32_t c = (byte >> sh) & 3u;
          /* code j of the group: byte j>>2 (word j>>4), bits (3-(j&3))*2 within the byte */
          const uint32_t wpos = (uint32_t)((j >> 2) & 3) * 8u + (3u - (uint32_t)(j & 3)) * 2u;
          out[j >> 4] = (out[j >> 4] & ~(3u << wpos)) | (c << wpos);
        }
      }
      *(uint4 *)(codes + (int64_t)r * ldc + (k0 >> 2) + 16 * half) =
          make_uint4(out[0], out[1], out[2], out[3]);
    }
    __syncthreads(); /* srec and soff are rewritten by the next tile */
  }
}

/*
 * sum over samples: codes[k][j] = code of sample samp[j] at kept SNP k; one row per kept
 * SNP, j over the nsamp samples; pad j and pad rows are 3.  One warp per SNP row: the
 * record is staged in shared memory (coalesced), then each lane gathers its 64-sample
 * groups from it.  Dynamic shared memory: warps x rlen bytes.
 */
__global__ void __launch_bounds__(256)
k_codes_by_snp(const uint8_t *__restrict__ geno, int64_t rlen, const int32_t *__restrict__ samp,
               int32_t nsamp, const int32_t *__restrict__ snprec, int32_t nk, int32_t nrows_pad,
               int64_t ldc, uint8_t *codes)
{
  extern __shared__ uint4 srec4[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  uint8_t *rec_s = (uint8_t *)(srec4 + (int64_t)warp * (rlen / 16));
  const int64_t groups = ldc / 16;
  for (int64_t k = (int64_t)blockIdx.x * nw + warp; k < nrows_pad; k += (int64_t)gridDim.x * nw) {
    if (k < nk) {
      const uint4 *src = (const uint4 *)(geno + (int64_t)snprec[k] * rlen);
      for (int64_t v = lane; v < rlen / 16; v += 32) ((uint4 *)rec_s)[v] = __ldg(src + v);
    }
    __syncwarp();
    for (int64_t gq = lane; gq < groups; gq += 32) {
      uint32_t out[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
      if (k < nk) {
#pragma unroll 8
        for (int j = 0; j < 64; ++j) {
          const int64_t q = gq * 64 + j;
          uint32_t c = 3u;
          if (q < nsamp) {
            const int32_t sidx = samp[q];
            c = (rec_s[sidx >> 2] >> ((3 - (sidx & 3)) * 2)) & 3u;
          }
          const uint32_t wpos = (uint32_t)((j >> 2) & 3) * 8u + (3u - (uint32_t)(j & 3)) * 2u;
          out[j >> 4] = (out[j >> 4] & ~(3u << wpos)) | (c << wpos);
        }
      }
      *(uint4 *)(codes + k * ldc + gq * 16) = make_uint4(out[0], out[1], out[2], out[3]);
    }
    __syncwarp();
  }
}

/*
 * per column c of P [nk][ldp] (FP64): running max of |P[k][c]| as its bit pattern (the
 * order of non-negative doubles), folded into mx[c] with atomicMax; threads keep a fixed
 * column so that a warp reads rows of P contiguously.  Several panels may fold into the
 * same mx (their joint exponent).
 */
__global__ void k_panel_absmax(const double *__restrict__ P, int64_t ldp, int32_t nk,
                               int32_t ncols, unsigned long long *mx)
{
  __shared__ unsigned long long smx[1024];
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) smx[c] = 0ull;
  __syncthreads();
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int64_t step = nthreads / ncols * ncols;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < step) {
    const int32_t c = (int32_t)(t % ncols);
    unsigned long long m = 0ull;
    const int64_t total = (int64_t)nk * ncols;
    for (int64_t idx = t; idx < total; idx += step) {
      const int64_t k = idx / ncols;
      const unsigned long long bits =
          (unsigned long long)__double_as_longlong(P[k * ldp + c]) & 0x7FFFFFFFFFFFFFFFull;
      m = bits > m ? bits : m;
    }
    if (m) atomicMax(smx + c, m);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < ncols; c += blockDim.x)
    if (smx[c]) atomicMax(mx + c, smx[c]);
}

/* exponent e_c with max|P| < 2^e_c (frexp), 0 for an all-zero column */
__global__ void k_panel_expo(const unsigned long long *mx, int32_t ncols, int32_t *expo)
{
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncols; c += gridDim.x * blockDim.x) {
    const double v = __longlong_as_double((long long)mx[c]);
    int e = 0;
    if (v > 0.0) frexp(v, &e); /* v = f 2^e, f in [0.5, 1) -> v < 2^e */
    expo[c] = e;
  }
}

/*
 * The four slices of x = sign P / 2^e_c (|x| < 1) in integer arithmetic (GB300's FP64 pipe is
 * narrow): N = rint(x 2^40) from the double's mantissa and exponent (round half to even),
 * then balanced base-1024 digits from the bottom, d_3, d_2, d_1 in [-512, 511] and
 * d_0 = the rest (|d_0| <= 1024 since |N| <= 2^40), so that x = sum_t d_t 1024^-(t+1) + O(2^-41).
 */
__device__ __forceinline__ void slice4(double v, int e, bool neg, int d[4])
{
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int E = (int)((bits >> 52) & 0x7FF);
  unsigned long long M = bits & 0xFFFFFFFFFFFFFull;
  /* |v| = M 2^(E' - 1075) with E' = max(E, 1); x 2^40 = M / 2^sh, sh >= 13 when |v| < 2^e */
  if (E) M |= 1ull << 52;
  const int sh = 1035 + e - (E ? E : 1);
  long long N = 0;
  if (M != 0 && sh < 64) {
    const int s = sh < 1 ? 1 : sh;
    unsigned long long q = M >> s;
    const unsigned long long rem = M & ((1ull << s) - 1), half = 1ull << (s - 1);
    if (rem > half || (rem == half && (q & 1ull))) ++q;
    N = (long long)q;
  }
  if (neg != (bool)(bits >> 63)) N = -N;
#pragma unroll
  for (int t = 3; t >= 1; --t) {
    int r = (int)(N & 1023);
    if (r >= 512) r -= 1024;
    d[t] = r;
    N = (N - r) >> 10; /* exact: N - r is a multiple of 1024 */
  }
  d[0] = (int)N;
}

/*
 * B[(4c+t)][koff + k] (fp16, row stride ldb elements) = slice t of sign P[k][c] / 2^e_c for
 * k < nk (pad k and pad rows are zero from a memset before).  A tile of 64 k x 32 columns is
 * read row-wise (coalesced) into shared memory and written as 128-byte rows of B.
 */
#define SL_K 64
#define SL_C 32
__global__ void __launch_bounds__(256)
k_panel_slices(const double *__restrict__ P, int64_t ldp, int32_t nk, int32_t ncols,
               const int32_t *__restrict__ expo, double sign, int64_t koff, __half *B, int64_t ldb)
{
  __shared__ double sp[SL_K][SL_C + 1];
  __shared__ __align__(16) __half ss[SL_C * 4][SL_K + 8];
  __shared__ int sexp[SL_C];
  const int tid = threadIdx.x;
  const int32_t kt0 = blockIdx.x * SL_K, ct0 = blockIdx.y * SL_C;
  const bool neg = sign < 0.0;
  if (tid < SL_C) {
    const int32_t c = ct0 + tid;
    sexp[tid] = c < ncols ? expo[c] : 0;
  }
  for (int i = tid; i < SL_K * SL_C; i += blockDim.x) {
    const int kk = i / SL_C, cc = i - kk * SL_C;
    const int32_t k = kt0 + kk, c = ct0 + cc;
    sp[kk][cc] = (k < nk && c < ncols) ? P[(int64_t)k * ldp + c] : 0.0;
  }
  __syncthreads();
  for (int i = tid; i < SL_K * SL_C; i += blockDim.x) {
    const int cc = i / SL_K, kk = i - cc * SL_K;
    int d[4];
    slice4(sp[kk][cc], sexp[cc], neg, d);
#pragma unroll
    for (int t = 0; t < 4; ++t) ss[4 * cc + t][kk] = __int2half_rn(d[t]);
  }
  __syncthreads();
  /* 128 output rows x 64 halves: 8 threads write one row's 128 bytes */
  for (int i = tid; i < SL_C * 4 * 8; i += blockDim.x) {
    const int o = i >> 3, seg = i & 7;
    const int32_t c = ct0 + (o >> 2);
    if (c >= ncols) continue;
    const int32_t k = kt0 + seg * 8;
    if (k >= nk) continue;
    __half *dst = B + (int64_t)(4 * ct0 + o) * ldb + koff + k;
    *(uint4 *)dst = *(const uint4 *)&ss[o][seg * 8];
  }
}

/* Y[r][c] = 2^e_c sum_t Z[r][4c+t] 1024^-(t+1) */
__global__ void k_panel_combine(const double *Z, int64_t ldz, int32_t nrows, int32_t ncols,
                                const int32_t *expo, double *Y, int64_t ldy,
                                const gp_tc_batch *db)
{
  if (db) nrows = db->nrows;
  int64_t total = (int64_t)nrows * ncols;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = idx / ncols;
    int32_t c = (int32_t)(idx - r * ncols);
    const double *z = Z + r * ldz + 4 * c;
    double s = ((z[0] * 0x1p-10 + z[1] * 0x1p-20) + z[2] * 0x1p-30) + z[3] * 0x1p-40;
    Y[r * ldy + c] = ldexp(s, expo[c]);
  }
}

/* ------------------------------------------------------------------------------------ */

static PFN_cuTensorMapEncodeTiled_v12000 tc_encode(gp_ctx *ctx)
{
  static PFN_cuTensorMapEncodeTiled_v12000 fn = NULL;
  if (fn) return fn;
  cudaDriverEntryPointQueryResult q;
  void *p = NULL;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                   cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
    gp_fail(ctx, GP_ERR_CUDA, "cuTensorMapEncodeTiled entry point not found");
    return NULL;
  }
  fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  return fn;
}

static int grid_cap(const gp_ctx *ctx, int64_t work, int per_block, int mult)
{
  int64_t g = (work + per_block - 1) / per_block;
  int64_t cap = (int64_t)ctx->num_sms * mult;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

int gp_tc_code_bytes(int sum_over_snps, int32_t nsamp, int32_t nk, int64_t *ldc, int32_t *rows_pad)
{
  const int32_t nrows = sum_over_snps ? nsamp : nk;
  const int32_t k0 = sum_over_snps ? nk : nsamp;
  *rows_pad = (nrows + XT - 1) / XT * XT;
  *ldc = (int64_t)((k0 + XK - 1) / XK) * XK / 4;
  return GP_OK;
}

int gp_tc_build_codes(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                      const int32_t *d_snprec, int32_t nk, uint8_t *codes, gp_tc_codes *out)
{
  int64_t ldc;
  int32_t nrows_pad;
  gp_tc_code_bytes(sum_over_snps, nsamp, nk, &ldc, &nrows_pad);
  if (sum_over_snps) {
    /* about 16 CTAs per SM in all; each walks the SNP tiles of its row block */
    const int64_t nkt = (ldc * 4 + CB_SNP - 1) / CB_SNP, nrb = (nrows_pad + CB_ROWS - 1) / CB_ROWS;
    int64_t gx = ((int64_t)ctx->num_sms * 16 + nrb - 1) / nrb;
    if (gx > nkt) gx = nkt;
    if (gx < 1) gx = 1;
    dim3 grid((unsigned)gx, (unsigned)nrb);
    k_codes_by_sample<<<grid, 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, d_samp, nsamp,
                                                     nrows_pad, d_snprec, nk, ldc, codes);
  } else {
    int warps = (int)((200 * 1024) / ctx->rlen_dev);
    if (warps > 8) warps = 8;
    if (warps < 1)
      return gp_fail(ctx, GP_ERR_ARG, "gp_tc_build_codes: records of %lld bytes are too long",
                     (long long)ctx->rlen_dev);
    const size_t smem = (size_t)warps * ctx->rlen_dev;
    GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_codes_by_snp));
    int blocks = (int)((nrows_pad + warps - 1) / warps);
    if (blocks > ctx->num_sms * 16) blocks = ctx->num_sms * 16;
    k_codes_by_snp<<<blocks, 32 * warps, smem, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, d_samp,
                                                              nsamp, d_snprec, nk, nrows_pad, ldc,
                                                              codes);
  }
  GP_LAUNCH_CHECK(ctx, "k_codes");
  out->codes = codes;
  out->ldc = ldc;
  out->row_map = NULL;
  out->nrows = sum_over_snps ? nsamp : nk;
  out->k0 = sum_over_snps ? nk : nsamp;
  return GP_OK;
}

size_t gp_tc_prepared_bytes(int npanels, int32_t ncols, int32_t k0)
{
  const int32_t kpad0 = (k0 + XK - 1) / XK * XK;
  const int32_t ncols4_pad = (4 * ncols + XT - 1) / XT * XT;
  return align256((size_t)ncols4_pad * kpad0 * npanels * 2) + align256((size_t)ncols * 16) + 256;
}

int gp_tc_prepare(gp_ctx *ctx, int npanels, const gp_tc_panel *pp, int32_t ncols, int32_t k0,
                  void *storage, gp_tc_prepared *out)
{
  if (npanels < 1 || npanels > 2 || ncols < 1 || ncols > 1024 || k0 < 1)
    return gp_fail(ctx, GP_ERR_ARG, "gp_tc_prepare: bad panel shape");
  const int32_t kb0 = (k0 + XK - 1) / XK, kpad0 = kb0 * XK;
  const int32_t ncols4 = 4 * ncols, ncols4_pad = (ncols4 + XT - 1) / XT * XT;
  const int64_t ldb = (int64_t)kpad0 * npanels;
  uint8_t *base = (uint8_t *)storage;
  __half *B = (__half *)base;
  uint8_t *ebase = base + align256((size_t)ncols4_pad * ldb * 2);
  unsigned long long *mx = (unsigned long long *)ebase; /* [ncols] joint max |P| bits */
  int32_t *expo = (int32_t *)(ebase + 8 * (size_t)ncols);
  GP_CUDA(ctx, cudaMemsetAsync(mx, 0, 8 * (size_t)ncols, ctx->stream));
  for (int p = 0; p < npanels; ++p) {
    int blocks = grid_cap(ctx, (int64_t)k0 * ncols, 256 * 16, 8);
    const int need = (ncols + 255) / 256;
    if (blocks < need) blocks = need;
    k_panel_absmax<<<blocks, 256, 0, ctx->stream>>>(pp[p].P, pp[p].ldp, k0, ncols, mx);
    GP_LAUNCH_CHECK(ctx, "k_panel_absmax");
  }
  k_panel_expo<<<(ncols + 255) / 256, 256, 0, ctx->stream>>>(mx, ncols, expo);
  GP_LAUNCH_CHECK(ctx, "k_panel_expo");
  GP_CUDA(ctx, cudaMemsetAsync(B, 0, (size_t)ncols4_pad * ldb * 2, ctx->stream));
  for (int p = 0; p < npanels; ++p) {
    dim3 sgrid((unsigned)((k0 + SL_K - 1) / SL_K), (unsigned)((ncols + SL_C - 1) / SL_C));
    k_panel_slices<<<sgrid, 256, 0, ctx->stream>>>(pp[p].P, pp[p].ldp, k0, ncols, expo,
                                                   pp[p].sign, (int64_t)p * kpad0, B, ldb);
    GP_LAUNCH_CHECK(ctx, "k_panel_slices");
  }
  PFN_cuTensorMapEncodeTiled_v12000 enc = tc_encode(ctx);
  if (!enc) return GP_ERR_CUDA;
  {
    cuuint64_t dims[2] = {(cuuint64_t)ldb, (cuuint64_t)ncols4_pad};
    cuuint64_t strides[1] = {(cuuint64_t)ldb * 2};
    cuuint32_t box[2] = {XK, XT};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&out->tmb, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, B, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return gp_fail(ctx, GP_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  }
  out->B = B;
  out->expo = expo;
  out->ncols = ncols;
  out->ncols4 = ncols4;
  out->ncols4_pad = ncols4_pad;
  out->npanels = npanels;
  out->kb0 = kb0;
  out->k0 = k0;
  out->ldb = ldb;
  out->lut_lo = pp[0].count ? LUT_COUNT : LUT_MASK;
  out->lut_hi = npanels > 1 ? (pp[1].count ? LUT_COUNT : LUT_MASK) : out->lut_lo;
  return GP_OK;
}

int gp_tc_apply(gp_ctx *ctx, const gp_tc_codes *A, const gp_tc_prepared *P, double *d_Y,
                int64_t ldy, int sync)
{
  const int32_t nrows = A->nrows;
  if (nrows < 1) return GP_OK;
  if (A->k0 != P->k0 || A->ldc < (int64_t)P->kb0 * XK / 4)
    return gp_fail(ctx, GP_ERR_ARG, "gp_tc_apply: code operand and panel disagree");
  const int64_t ldz = P->ncols4_pad;
  double *Z;
  int rc = gp_scratch5(ctx, (size_t)nrows * ldz * 8 + 256, (void **)&Z);
  if (rc) return rc;
  int *d_err = ctx->d_err;
  if (sync) GP_CUDA(ctx, cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  GP_CUDA(ctx, cudaMemsetAsync(Z, 0, (size_t)nrows * ldz * 8, ctx->stream));
  GP_CUDA(ctx, cudaFuncSetAttribute(k_geno_panel_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    X_SMEM));
  const int32_t nkb = P->kb0 * P->npanels;
  const int32_t nrt = (nrows + XT - 1) / XT, nct = P->ncols4_pad / XT;
  int32_t tiles = nrt * nct;
  int32_t ksplit = 1;
  while (tiles * ksplit < 2 * ctx->num_sms && ksplit * 4 <= nkb) ksplit *= 2;
  /* keep each work item's k range below 2^19 so that int32 sums stay exact */
  while ((int64_t)((nkb + ksplit - 1) / ksplit) * XK > (1 << 19)) ksplit *= 2;
  int32_t nitems = tiles * ksplit;
  int grid = nitems < ctx->num_sms ? nitems : ctx->num_sms;
  k_geno_panel_tc<<<grid, X_THREADS, X_SMEM, ctx->stream>>>(P->tmb, A->codes, A->ldc, A->row_map,
                                                           nrows, P->ncols4, nkb, P->kb0, P->kb0,
                                                           P->lut_lo, P->lut_hi, ksplit, Z, ldz,
                                                           d_err, NULL);
  GP_LAUNCH_CHECK(ctx, "k_geno_panel_tc");
  {
    int64_t work = (int64_t)nrows * P->ncols;
    k_panel_combine<<<grid_cap(ctx, work, 256, 32), 256, 0, ctx->stream>>>(Z, ldz, nrows, P->ncols,
                                                                            P->expo, d_Y, ldy, NULL);
    GP_LAUNCH_CHECK(ctx, "k_panel_combine");
  }
  if (!sync) return GP_OK;
  int herr = 0;
  GP_CUDA(ctx, gp_memcpy(ctx, &herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (herr) return gp_fail(ctx, GP_ERR_TIMEOUT, "tensor-core product wait timed out (code %d)", herr);
  return GP_OK;
}

/* Z[r][c] = 0 for the batch's rows */
__global__ void k_zero_batch_rows(double *Z, int64_t ldz, const gp_tc_batch *db)
{
  const int64_t total = (int64_t)db->nrows * ldz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    Z[i] = 0.0;
}

int gp_tc_apply_dev(gp_ctx *ctx, const gp_tc_batch *db, int32_t max_rows, int64_t ldc,
                    const gp_tc_prepared *P, double *Z, double *d_Y, int64_t ldy)
{
  if (max_rows < 1) return GP_OK;
  if (ldc < (int64_t)P->kb0 * XK / 4)
    return gp_fail(ctx, GP_ERR_ARG, "gp_tc_apply_dev: code rows shorter than the panel");
  const int64_t ldz = P->ncols4_pad;
  k_zero_batch_rows<<<grid_cap(ctx, (int64_t)max_rows * ldz, 256, 8), 256, 0, ctx->stream>>>(
      Z, ldz, db);
  GP_LAUNCH_CHECK(ctx, "k_zero_batch_rows");
  GP_CUDA(ctx, cudaFuncSetAttribute(k_geno_panel_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    X_SMEM));
  const int32_t nkb = P->kb0 * P->npanels;
  /* every SM: the kernel takes the batch's row count, and with it its work items, from db */
  k_geno_panel_tc<<<ctx->num_sms, X_THREADS, X_SMEM, ctx->stream>>>(
      P->tmb, NULL, ldc, NULL, 0, P->ncols4, nkb, P->kb0, P->kb0, P->lut_lo, P->lut_hi, 1, Z, ldz,
      ctx->d_err, db);
  GP_LAUNCH_CHECK(ctx, "k_geno_panel_tc");
  k_panel_combine<<<grid_cap(ctx, (int64_t)max_rows * P->ncols, 256, 32), 256, 0, ctx->stream>>>(
      Z, ldz, 0, P->ncols, P->expo, d_Y, ldy, db);
  GP_LAUNCH_CHECK(ctx, "k_panel_combine");
  return GP_OK;
}

int gp_geno_panel_tc_codes(gp_ctx *ctx, const gp_tc_codes *A, int npanels, const gp_tc_panel *pp,
                           int32_t ncols, double *d_Y, int64_t ldy)
{
  if (A->nrows < 1 || A->k0 < 1) return GP_OK;
  uint8_t *storage;
  int rc = gp_scratch2(ctx, gp_tc_prepared_bytes(npanels, ncols, A->k0), (void **)&storage);
  if (rc) return rc;
  gp_tc_prepared P;
  rc = gp_tc_prepare(ctx, npanels, pp, ncols, A->k0, storage, &P);
  if (rc) return rc;
  return gp_tc_apply(ctx, A, &P, d_Y, ldy, 1);
}

int gp_tc_codes_for(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                    const int32_t *d_snprec, int32_t nk, gp_tc_codes *out)
{
  const int current_rows = sum_over_snps && d_samp == ctx->d_rows && nsamp == ctx->nrows &&
                           nk == ctx->nkept;
  if (current_rows && ctx->codes4_rows) {
    /* the sample-major codes of the current rows are still in place */
    int64_t ldc;
    int32_t rows_pad;
    gp_tc_code_bytes(1, nsamp, nk, &ldc, &rows_pad);
    out->codes = (uint8_t *)ctx->d_scratch4;
    out->ldc = ldc;
    out->row_map = NULL;
    out->nrows = nsamp;
    out->k0 = nk;
    return GP_OK;
  }
  if (!sum_over_snps && nsamp == ctx->nind_all) {
    /* every sample in order: the resident records are the SNP-major operand */
    out->codes = ctx->d_geno;
    out->ldc = ctx->rlen_dev;
    out->row_map = d_snprec;
    out->nrows = nk;
    out->k0 = nsamp;
    return GP_OK;
  }
  int64_t ldc;
  int32_t rows_pad;
  gp_tc_code_bytes(sum_over_snps, nsamp, nk, &ldc, &rows_pad);
  uint8_t *codes;
  int rc = gp_scratch4(ctx, (size_t)rows_pad * ldc + 256, (void **)&codes);
  if (rc) return rc;
  rc = gp_tc_build_codes(ctx, sum_over_snps, d_samp, nsamp, d_snprec, nk, codes, out);
  if (!rc && current_rows) ctx->codes4_rows = 1;
  return rc;
}

int gp_geno_panel_tc(gp_ctx *ctx, int sum_over_snps, const int32_t *d_samp, int32_t nsamp,
                     const int32_t *d_snprec, int32_t nk, int npanels, const gp_tc_panel *pp,
                     int32_t ncols, double *d_Y, int64_t ldy)
{
  if ((sum_over_snps ? nsamp : nk) < 1 || (sum_over_snps ? nk : nsamp) < 1) return GP_OK;
  gp_tc_codes A;
  int rc = gp_tc_codes_for(ctx, sum_over_snps, d_samp, nsamp, d_snprec, nk, &A);
  if (rc) return rc;
  return gp_geno_panel_tc_codes(ctx, &A, npanels, pp, ncols, d_Y, ldy);
}
