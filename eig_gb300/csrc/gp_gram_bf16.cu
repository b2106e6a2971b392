/*
 * Split-BF16 Gram on the 5th-generation tensor cores (tcgen05), replacing the reference's
 * XTX accumulation (domult_increment_lookup / block_increment_binary,
 * src/eigensrc/smartpca.c:3361-3495) for GP_PREC_SPLIT_BF16.
 *
 * Each normalised value v (the FP64 table entry of its SNP and genotype code) is split into
 * hi = r(v) and lo = r(v - hi) in a 16-bit format (bf16 or fp16).  XTX = Xhi Xhi^T +
 * Xhi Xlo^T + Xlo Xhi^T (+ Xlo Xlo^T with 4 MMAs): tcgen05 MMAs with FP32 accumulation in
 * TMEM over a short SNP chunk (128 SNPs by default: the tensor core's FP32 accumulation
 * truncates, so its error grows with the chunk depth), chunk sums added in FP32 registers
 * (round to nearest) for a few chunks, then folded into a per-element running sum held in
 * TMEM as an FP32 (hi, lo) pair with TwoSum (~48 bits), which stands in for FP64
 * accumulation at FP32 speed (GB300's FP64 rate is a small fraction of its FP32 rate); the
 * tile is written out in FP64.
 *
 * Data layout in HBM: Xhi and Xlo as row-major [Npad][Kc] bf16 (samples x kept SNPs of the
 * current super-chunk), written by k_split_transpose from the packed records; the Gram
 * kernel reads them with TMA as 128-row x 64-SNP boxes in the 128-byte swizzle.
 *
 * Kernel structure (persistent, one CTA per SM, 18 warps):
 *   warp 0      TMA producer: per k-block of 64 SNPs four 16 KB boxes (A hi/lo, B hi/lo)
 *               into a 3-stage shared-memory ring;
 *   warp 1      allocates 512 TMEM columns; one thread issues 12 (or 16) tcgen05.mma
 *               (128x128x16) per k-block into FP32 accumulator buffer (chunk & 1),
 *               columns 0-255;
 *   warps 2-17  epilogue: at the end of each chunk read the FP32 buffer (tcgen05.ld),
 *               release it and add it into registers; every GP_FOLD chunks fold those into
 *               the (hi, lo) running sums in TMEM columns 256-511; after the last chunk of a
 *               tile write the tile to the Gram in FP64.
 * Tiles are the 128x128 blocks of the lower triangle, distributed round-robin over CTAs, or
 * over clusters: four CTAs on a 2 x 2 block of tiles (each loads one box of its tile row and
 * one of its tile column and multicasts it to the two CTAs that share it: half the boxes of
 * the one-CTA kernel) or two CTAs on two tiles of a row (the row's boxes multicast: three
 * quarters).  A stage is then released when every CTA of the cluster has read it
 * (tcgen05.commit multicast to each CTA's empty barrier).
 */
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <stdlib.h>

#include "gp_internal.h"
#include "gp_tc.cuh"

#define BT 128          /* tile edge (rows of A and B) */
#define BK 64           /* SNPs per k-block (128 bytes of bf16) */
#define NSTAGE 3
#define BOX_BYTES (BT * BK * 2)
#define STAGE_BYTES (4 * BOX_BYTES)
#ifndef EPI_COLS
#define EPI_COLS 32 /* tile columns per epilogue thread */
#endif
#ifndef GP_FOLD
#define GP_FOLD 8   /* chunks summed in FP32 registers before the TwoSum fold */
#endif
#define GRAM_THREADS (64 + 32 * 4 * (128 / EPI_COLS)) /* producer + MMA + epilogue warps */
#define GRAM_SMEM (NSTAGE * STAGE_BYTES + 1024 + 256)

/* error codes recorded by the kernel */
#define GP_KERR_TIMEOUT_FULL 1
#define GP_KERR_TIMEOUT_EMPTY 2
#define GP_KERR_TIMEOUT_ACCF 3
#define GP_KERR_TIMEOUT_ACCE 4
#define GP_KERR_TIMEOUT_SYNC 5
#define GP_KERR_CLUSTER 6 /* launched without clusters of the kernel's size */
#define GRAM_SYNC_KB 64 /* k-blocks between the producers' lockstep points */

__device__ __forceinline__ int32_t tri_root(int32_t t)
{
  int32_t i = (int32_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  while (i * (i + 1) / 2 > t) --i;
  return i;
}

/*
 * Tile t of the lower triangle of nt x nt tiles, in groups: the tile grid is cut into
 * GRAM_GROUP x GRAM_GROUP blocks (lower triangle of blocks, row by row), tiles row by row
 * inside a block.  The CTAs that run at the same time then hold tiles of a few row blocks
 * and walk the SNPs at the same pace, so the operand boxes they load are shared in L2
 * instead of being read from HBM once per tile.
 */
#define GRAM_GROUP 12
/* element t of the lower triangle of an nt x nt grid walked in gs x gs groups */
__device__ __forceinline__ void tri_tile_group(int32_t t, int32_t nt, int32_t gs, int32_t *bi,
                                               int32_t *bj)
{
  const int32_t ng = (nt + gs - 1) / gs;
  for (int32_t gi = 0; gi < ng; ++gi) {
    const int32_t r0 = gi * gs, nr = min(nt, r0 + gs) - r0;
    for (int32_t gj = 0; gj <= gi; ++gj) {
      const int32_t c0 = gj * gs, nc = min(nt, c0 + gs) - c0;
      const int32_t cnt = gi == gj ? nr * (nr + 1) / 2 : nr * nc;
      if (t < cnt) {
        if (gi == gj) {
          const int32_t i = tri_root(t);
          *bi = r0 + i;
          *bj = c0 + t - i * (i + 1) / 2;
        } else {
          *bi = r0 + t / nc;
          *bj = c0 + t % nc;
        }
        return;
      }
      t -= cnt;
    }
  }
  *bi = *bj = 0; /* not reached for t < nt (nt + 1) / 2 */
}

__device__ __forceinline__ void tri_tile(int32_t t, int32_t nt, int32_t *bi, int32_t *bj)
{
  const int32_t ng = (nt + GRAM_GROUP - 1) / GRAM_GROUP;
  for (int32_t gi = 0; gi < ng; ++gi) {
    const int32_t r0 = gi * GRAM_GROUP, nr = min(nt, r0 + GRAM_GROUP) - r0;
    for (int32_t gj = 0; gj <= gi; ++gj) {
      const int32_t c0 = gj * GRAM_GROUP, nc = min(nt, c0 + GRAM_GROUP) - c0;
      const int32_t cnt = gi == gj ? nr * (nr + 1) / 2 : nr * nc;
      if (t < cnt) {
        if (gi == gj) {
          const int32_t i = tri_root(t);
          *bi = r0 + i;
          *bj = c0 + t - i * (i + 1) / 2;
        } else {
          *bi = r0 + t / nc;
          *bj = c0 + t % nc;
        }
        return;
      }
      t -= cnt;
    }
  }
  *bi = *bj = 0; /* not reached for t < ntiles */
}

/*
 * Pair p of tiles for a cluster of two CTAs: the tiles of one tile row are taken two at a time
 * (columns 2q, 2q+1 of the row inside its group block), so the pair shares the row block bi
 * (the A operand).  bj1 = -1 when the row has an odd count and p is its last pair.
 */
__device__ __forceinline__ void tri_pair(int32_t p, int32_t nt, int32_t *bi, int32_t *bj0,
                                         int32_t *bj1)
{
  const int32_t ng = (nt + GRAM_GROUP - 1) / GRAM_GROUP;
  for (int32_t gi = 0; gi < ng; ++gi) {
    const int32_t r0 = gi * GRAM_GROUP, nr = min(nt, r0 + GRAM_GROUP) - r0;
    for (int32_t gj = 0; gj <= gi; ++gj) {
      const int32_t c0 = gj * GRAM_GROUP, nc = min(nt, c0 + GRAM_GROUP) - c0;
      for (int32_t lr = 0; lr < nr; ++lr) {
        const int32_t len = gi == gj ? lr + 1 : nc;
        const int32_t np = (len + 1) / 2;
        if (p < np) {
          *bi = r0 + lr;
          *bj0 = c0 + 2 * p;
          *bj1 = 2 * p + 1 < len ? c0 + 2 * p + 1 : -1;
          return;
        }
        p -= np;
      }
    }
  }
  *bi = *bj0 = 0; /* not reached for p < npairs */
  *bj1 = -1;
}

/*
 * Quad w: a 2 x 2 block of tiles (tile rows 2I, 2I+1, tile columns 2J, 2J+1, J <= I) for a
 * cluster of four CTAs, quads in GRAM_GROUP/2-square groups (lower triangle of groups, row by
 * row inside a group) like the tiles of tri_tile.
 */
__device__ __forceinline__ void tri_quad(int32_t w, int32_t nq, int32_t *qi, int32_t *qj)
{
  tri_tile_group(w, nq, GRAM_GROUP / 2, qi, qj);
}

/*
 * The tile of work item w for this CTA (cluster rank `rank`): CL = 1 a tile; CL = 2 the
 * rank's tile of pair w (the second CTA of an odd pair computes the first tile again); CL = 4
 * tile (2I + rank/2, 2J + rank%2) of quad w.  *write is false for a stand-in tile (a second
 * tile the pair does not have, or a quad position outside the lower triangle or the matrix);
 * *arow / *bcol are the tile row and column whose boxes the CTA loads (in the matrix always).
 */
template <int CL>
__device__ __forceinline__ void gram_work(int32_t w, int32_t nt, uint32_t rank, int32_t *bi,
                                          int32_t *bj, bool *write)
{
  if (CL == 1) {
    tri_tile(w, nt, bi, bj);
    *write = true;
  } else if (CL == 2) {
    int32_t j0, j1;
    tri_pair(w, nt, bi, &j0, &j1);
    *bj = (rank == 0 || j1 < 0) ? j0 : j1;
    *write = rank == 0 || j1 >= 0;
  } else {
    int32_t qi, qj;
    tri_quad(w, (nt + 1) / 2, &qi, &qj);
    const int32_t ti = 2 * qi + (int32_t)(rank >> 1), tj = 2 * qj + (int32_t)(rank & 1);
    *write = ti < nt && tj < nt && tj <= ti;
    *bi = ti < nt ? ti : 2 * qi;
    *bj = tj < nt ? tj : 2 * qj;
  }
}

/*
 * grams: XTX (n x n row-major FP64); accumulate != 0 adds to the values already there
 * (super-chunks after the first).  nkb = k-blocks of this super-chunk; chunk_kb = k-blocks
 * per FP32 accumulation chunk.
 */
template <int FP16, int NMMA, int CL>
__global__ void __launch_bounds__(GRAM_THREADS, 1)
k_gram_split(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo,
                  int32_t nwork, int32_t nt_rows, int32_t nkb, int32_t chunk_kb, double *xtx,
                  int32_t n, int32_t accumulate, unsigned *sync_ctr, int *err)
{
  /* CL = 2: clusters of two CTAs computing two tiles of one tile row; the row block's boxes
   * (A hi and lo) are multicast to both, one box by each CTA.  CL = 4: clusters of four CTAs
   * computing a 2 x 2 block of tiles; each CTA loads one of the two boxes of its tile row
   * (multicast to the row's two CTAs) and one of the two boxes of its tile column
   * (multicast to the column's two CTAs).  A stage is released when every CTA's MMAs of the
   * cluster have read it. */
  /* a cluster kernel run without clusters of its size (for instance a launch that lost the
   * cluster attribute) would multicast to CTAs that do not exist: it refuses to run */
  if (CL > 1 && cluster_nctarank() != (uint32_t)CL) {
    if (threadIdx.x == 0) atomicExch(err, GP_KERR_CLUSTER);
    return;
  }
  const uint32_t rank = CL > 1 ? cluster_ctarank() : 0u;
  const int32_t w0 = CL > 1 ? (int32_t)cluster_id_x() : (int32_t)blockIdx.x;
  const int32_t wstride = CL > 1 ? (int32_t)cluster_count_x() : (int32_t)gridDim.x;
  const uint16_t all_mask = (uint16_t)((1u << CL) - 1u);
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bars = (uint64_t *)(smem + NSTAGE * STAGE_BYTES);
  uint64_t *full = bars;                 /* [NSTAGE] */
  uint64_t *empty = bars + NSTAGE;       /* [NSTAGE] */
  uint64_t *accf = bars + 2 * NSTAGE;    /* [2] */
  uint64_t *acce = bars + 2 * NSTAGE + 2;/* [2] */
  uint64_t *drain = bars + 2 * NSTAGE + 4; /* abort path: wait for issued MMAs */
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * NSTAGE + 5);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CL);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 4 * (128 / EPI_COLS));
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 0 && lane == 0) {
    tma_prefetch_desc(&tm_hi);
    tma_prefetch_desc(&tm_lo);
  }
  if (warp == 1) tmem_alloc(tmem_slot, 512);
  tc_fence_before();
  __syncthreads();
  if (CL > 1) cluster_sync_all(); /* the peers' barriers are initialised before any multicast */
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int32_t nchunk = (nkb + chunk_kb - 1) / chunk_kb;

  if (warp == 0) {
    /* ---------------- TMA producer ---------------- */
    if (lane == 0) {
      uint32_t it = 0;
      const int32_t nsync = (nkb + GRAM_SYNC_KB - 1) / GRAM_SYNC_KB;
      for (int32_t t = w0; t < nwork && !*abort_flag; t += wstride) {
        int32_t bi, bj;
        bool wr;
        gram_work<CL>(t, nt_rows, rank, &bi, &bj, &wr);
        /* the CTAs of one wave (work items t / wstride) meet every GRAM_SYNC_KB k-blocks, so
         * that the boxes one of them loads are still in L2 when the others need them */
        const int32_t wave = t / wstride;
        const unsigned wave_n = (unsigned)(min(wstride, nwork - wave * wstride) * CL);
        for (int32_t kb = 0; kb < nkb; ++kb, ++it) {
          if (kb > 0 && kb % GRAM_SYNC_KB == 0) {
            unsigned *ctr = sync_ctr + (int64_t)wave * nsync + kb / GRAM_SYNC_KB;
            atomicAdd(ctr, 1u);
            volatile unsigned *vc = ctr;
            const uint64_t t0 = globaltimer_ns();
            bool ok = true;
            while (*vc < wave_n) {
              if (*abort_flag) {
                ok = false;
                break;
              }
              if (globaltimer_ns() - t0 > GP_WAIT_NS) {
                atomicExch(err, GP_KERR_TIMEOUT_SYNC);
                *abort_flag = 1;
                ok = false;
                break;
              }
            }
            if (!ok) break;
          }
          uint32_t s = it % NSTAGE, ph = (it / NSTAGE) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag, err, GP_KERR_TIMEOUT_EMPTY)) break;
          uint8_t *st = smem + s * STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
          if (CL == 4) {
            /* rank = 2 a + b: row a's box (hi for b = 0, lo for b = 1) to ranks 2a, 2a+1;
             * column b's box (hi for a = 0, lo for a = 1) to ranks b, b+2 */
            const uint32_t a = rank >> 1, b = rank & 1u;
            const uint16_t rmask = (uint16_t)(3u << (2 * a)), cmask = (uint16_t)(5u << b);
            tma_load_2d_mc(st + b * BOX_BYTES, b ? &tm_lo : &tm_hi, &full[s], kb * BK, bi * BT,
                           rmask);
            tma_load_2d_mc(st + (2 + a) * BOX_BYTES, a ? &tm_lo : &tm_hi, &full[s], kb * BK,
                           bj * BT, cmask);
          } else {
            if (CL == 2) {
              /* A hi from rank 0 and A lo from rank 1, each into both CTAs */
              if (rank == 0)
                tma_load_2d_mc(st, &tm_hi, &full[s], kb * BK, bi * BT, (uint16_t)3);
              else
                tma_load_2d_mc(st + BOX_BYTES, &tm_lo, &full[s], kb * BK, bi * BT, (uint16_t)3);
            } else {
              tma_load_2d(st, &tm_hi, &full[s], kb * BK, bi * BT);
              tma_load_2d(st + BOX_BYTES, &tm_lo, &full[s], kb * BK, bi * BT);
            }
            tma_load_2d(st + 2 * BOX_BYTES, &tm_hi, &full[s], kb * BK, bj * BT);
            tma_load_2d(st + 3 * BOX_BYTES, &tm_lo, &full[s], kb * BK, bj * BT);
          }
        }
      }
      if (*abort_flag) {
        /* copies already issued must land before the CTA exits (bounded) */
        uint32_t last = it < NSTAGE ? it : NSTAGE;
        for (uint32_t j = it - last; j < it; ++j) {
          uint64_t t0 = globaltimer_ns();
          while (!mbar_try_wait(&full[j % NSTAGE], (j / NSTAGE) & 1u) &&
                 globaltimer_ns() - t0 < GP_WAIT_NS) {
          }
        }
      }
    }
  } else if (warp == 1) {
    /* ---------------- MMA issuer ---------------- */
    if (lane == 0) {
      const uint32_t idesc = FP16 ? idesc_f16_f32(BT, BT) : idesc_bf16_f32(BT, BT);
      uint32_t it = 0, chunk = 0;
      bool ok = true;
      for (int32_t t = w0; t < nwork && ok; t += wstride) {
        for (int32_t c = 0; c < nchunk && ok; ++c, ++chunk) {
          uint32_t buf = chunk & 1u, use = chunk >> 1;
          if (!mbar_wait(&acce[buf], (use & 1u) ^ 1u, abort_flag, err, GP_KERR_TIMEOUT_ACCE)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + buf * BT;
          int32_t kb0 = c * chunk_kb, kb1 = kb0 + chunk_kb < nkb ? kb0 + chunk_kb : nkb;
          for (int32_t kb = kb0; kb < kb1; ++kb, ++it) {
            uint32_t s = it % NSTAGE, ph = (it / NSTAGE) & 1u;
            if (!mbar_wait(&full[s], ph, abort_flag, err, GP_KERR_TIMEOUT_FULL)) {
              ok = false;
              break;
            }
            tc_fence_after();
            uint32_t base = smem_u32(smem + s * STAGE_BYTES);
            uint64_t ahi = sdesc_k128(base), alo = sdesc_k128(base + BOX_BYTES);
            uint64_t bhi = sdesc_k128(base + 2 * BOX_BYTES), blo = sdesc_k128(base + 3 * BOX_BYTES);
#pragma unroll
            for (int k = 0; k < BK / 16; ++k) {
              /* +32 bytes along K per 16 bf16 = +2 in the 16-byte address field */
              uint64_t o = (uint64_t)(2 * k);
              uint32_t acc0 = (kb > kb0 || k > 0) ? 1u : 0u;
              umma_bf16(d, ahi + o, bhi + o, idesc, acc0);
              umma_bf16(d, ahi + o, blo + o, idesc, 1u);
              umma_bf16(d, alo + o, bhi + o, idesc, 1u);
              if (NMMA == 4) umma_bf16(d, alo + o, blo + o, idesc, 1u);
            }
            if (CL > 1)
              umma_commit_mc(&empty[s], all_mask); /* this CTA has read the stage */
            else
              umma_commit(&empty[s]);
          }
          if (!ok) break;
          umma_commit(&accf[buf]);
        }
      }
    }
  } else {
    /* ---------------- epilogue (warps 2..17) ----------------
     * Warp w reads TMEM lanes 32*(w%4)..+31 (its row quarter); the four warps of a quarter
     * take EPI_COLS columns each.  Three levels of accumulation:
     *   tensor core  FP32 over one chunk (chunk_kb k-blocks) in TMEM buffer (chunk & 1);
     *   registers    FP32 (round-to-nearest) sum of GP_FOLD chunks, A[];
     *   TMEM         running sum as an FP32 (hi, lo) pair updated with TwoSum (~48 bits),
     *                columns 256+col (hi) and 384+col (lo), written out in FP64 per tile.
     * No FP64 arithmetic on the per-chunk path (GB300's FP64 rate is low). */
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const int col0 = ((warp - 2) >> 2) * EPI_COLS;
    const uint32_t lane_addr = (uint32_t)(q * 32) << 16;
    const uint32_t t_acc = tmem + lane_addr;
    uint32_t chunk = 0;
    bool ok = true;
    for (int32_t t = w0; t < nwork && ok; t += wstride) {
      int32_t bi, bj;
      bool wr;
      gram_work<CL>(t, nt_rows, rank, &bi, &bj, &wr);
      const int32_t gi = bi * BT + row;
      const int32_t gj0 = bj * BT + col0;
      float A[EPI_COLS];
      {
        uint32_t z[16];
#pragma unroll
        for (int v = 0; v < 16; ++v) z[v] = 0u;
#pragma unroll
        for (int g = 0; g < EPI_COLS / 16; ++g) {
          tmem_st16(t_acc + 256 + col0 + 16 * g, z);
          tmem_st16(t_acc + 384 + col0 + 16 * g, z);
        }
        tmem_wait_st();
      }
#pragma unroll
      for (int u = 0; u < EPI_COLS; ++u) A[u] = 0.f;
      for (int32_t c = 0; c < nchunk; ++c, ++chunk) {
        uint32_t buf = chunk & 1u, use = chunk >> 1;
        bool got = mbar_wait(&accf[buf], use & 1u, abort_flag, err, GP_KERR_TIMEOUT_ACCF);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int g = 0; g < EPI_COLS / 16; ++g) {
          uint32_t f[16];
          tmem_ld16(t_acc + buf * BT + col0 + 16 * g, f);
          tmem_wait_ld();
#pragma unroll
          for (int v = 0; v < 16; ++v) A[16 * g + v] = __fadd_rn(A[16 * g + v], __uint_as_float(f[v]));
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[buf]); /* buffer free: the MMA may reuse it */
        if ((c + 1) % GP_FOLD == 0 || c + 1 == nchunk) {
          /* fold A into the (hi, lo) running sum with TwoSum */
#pragma unroll
          for (int g = 0; g < EPI_COLS / 16; ++g) {
            uint32_t hs[16], ls[16];
            tmem_ld16(t_acc + 256 + col0 + 16 * g, hs);
            tmem_ld16(t_acc + 384 + col0 + 16 * g, ls);
            tmem_wait_ld();
#pragma unroll
            for (int v = 0; v < 16; ++v) {
              float Sv = __uint_as_float(hs[v]), x = A[16 * g + v];
              float s1 = __fadd_rn(Sv, x);
              float bp = __fsub_rn(s1, Sv);
              float e = __fadd_rn(__fsub_rn(Sv, __fsub_rn(s1, bp)), __fsub_rn(x, bp));
              hs[v] = __float_as_uint(s1);
              ls[v] = __float_as_uint(__fadd_rn(__uint_as_float(ls[v]), e));
              A[16 * g + v] = 0.f;
            }
            tmem_st16(t_acc + 256 + col0 + 16 * g, hs);
            tmem_st16(t_acc + 384 + col0 + 16 * g, ls);
          }
          tmem_wait_st();
        }
      }
      if (!ok) break;
      /* the tile -> Gram rows in FP64 (super-chunks after the first add to what is there) */
      double *orow = xtx + (int64_t)gi * n;
#pragma unroll
      for (int g = 0; g < EPI_COLS / 16; ++g) {
        uint32_t hs[16], ls[16];
        tmem_ld16(t_acc + 256 + col0 + 16 * g, hs);
        tmem_ld16(t_acc + 384 + col0 + 16 * g, ls);
        tmem_wait_ld();
        if (wr && gi < n) {
          for (int v = 0; v < 16; ++v) {
            int32_t gj = gj0 + 16 * g + v;
            if (gj < n) {
              double x = (double)__uint_as_float(hs[v]) + (double)__uint_as_float(ls[v]);
              orow[gj] = accumulate ? orow[gj] + x : x;
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1 && lane == 0 && (CL > 1 || *abort_flag)) {
    /* let MMAs already issued finish (and, in a pair, their arrivals on the peer's
     * barriers land) before the columns are released and the CTA leaves */
    umma_commit(drain);
    uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(drain, 0) && globaltimer_ns() - t0 < GP_WAIT_NS) {
    }
  }
  __syncthreads();
  if (CL > 1) cluster_sync_all(); /* no multicast or remote arrive targets a CTA that has left */
  if (warp == 1) {
    __syncwarp();
    tmem_dealloc(tmem, 512);
  }
}

/* ------------------------------------------------------------------------------------ */
/* split materialisation                                                                  */

/* per kept column: (hi, lo) 16-bit pairs (bf16 or fp16) for codes 0..3 packed as
 * 4 x uint32 (lo << 16 | hi); hi = round(v), lo = round(v - hi) */
template <int FP16>
__global__ void k_split_tables(const int32_t *kept, int32_t nkept, const double *vtab,
                               uint32_t *split)
{
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nkept; k += gridDim.x * blockDim.x) {
    int32_t c = kept[k];
    for (int g = 0; g < 4; ++g) {
      double v = vtab[4 * c + g];
      uint32_t h, l;
      if (FP16) {
        __half hi = __double2half(v);
        __half lo = __double2half(v - (double)__half2float(hi));
        h = (uint32_t)__half_as_ushort(hi);
        l = (uint32_t)__half_as_ushort(lo);
      } else {
        __nv_bfloat16 hi = __double2bfloat16(v);
        __nv_bfloat16 lo = __double2bfloat16(v - (double)__bfloat162float(hi));
        h = (uint32_t)__bfloat16_as_ushort(hi);
        l = (uint32_t)__bfloat16_as_ushort(lo);
      }
      split[4 * k + g] = h | (l << 16);
    }
  }
}

/*
 * Xhi/Xlo [npad][kc] for kept columns [k0, k0 + kc), rows >= nrows and columns >= nkept zero,
 * tile by tile through shared memory (a transpose of the SNP-major records):
 * CTA (kt, rt) covers 64 kept SNPs x 256 output rows.  When the tile's samples span at most
 * 256 record bytes (always when the rows are all samples or a subset with few gaps) the 64
 * records' byte ranges are read once, coalesced, into shared memory; each thread then writes
 * whole 16-byte groups so that a warp stores four 128-byte row segments.  Wider spans (sparse
 * sample subsets) read the bytes from global memory per thread.
 */
#define MT_SNP 64
#define MT_ROWS 256
#define MT_SPAN 256
#define MT_PITCH_W (MT_SPAN / 4 + 1) /* 65 words: rows one bank apart */
__global__ void __launch_bounds__(256)
k_split_transpose(const uint8_t *__restrict__ geno, int64_t rlen, const int32_t *__restrict__ rows,
                  int32_t nrows, const int32_t *__restrict__ cols, const int32_t *__restrict__ kept,
                  int32_t nkept, const uint32_t *__restrict__ split, int32_t k0, int32_t kc,
                  int32_t npad, __nv_bfloat16 *xhi, __nv_bfloat16 *xlo)
{
  __shared__ uint32_t srec[MT_SNP][MT_PITCH_W];
  __shared__ uint32_t stab[MT_SNP][4];
  __shared__ int64_t srecoff[MT_SNP];
  const int tid = threadIdx.x;
  const int32_t kt = blockIdx.x, r0 = blockIdx.y * MT_ROWS;
  const int32_t kbase = k0 + kt * MT_SNP;
  int32_t base = 0, span = 0;
  if (r0 < nrows) {
    const int32_t rl = (r0 + MT_ROWS < nrows ? r0 + MT_ROWS : nrows) - 1;
    base = (rows[r0] >> 2) & ~15;
    span = (rows[rl] >> 2) - base + 1;
  }
  const bool fast = span <= MT_SPAN;
  if (tid < MT_SNP) {
    const int32_t k = kbase + tid;
    srecoff[tid] = k < nkept ? (int64_t)cols[kept[k]] * rlen : -1;
  }
  {
    const int u = tid >> 2, g = tid & 3;
    const int32_t k = kbase + u;
    stab[u][g] = k < nkept ? __ldg(split + 4 * k + g) : 0u;
  }
  __syncthreads();
  if (fast && span > 0) {
    const int nvec = (span + 15) >> 4;
    for (int i = tid; i < MT_SNP * nvec; i += blockDim.x) {
      const int u = i / nvec, v = i - u * nvec;
      uint4 val = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
      if (srecoff[u] >= 0) val = __ldg((const uint4 *)(geno + srecoff[u] + base + 16 * v));
      srec[u][4 * v] = val.x;
      srec[u][4 * v + 1] = val.y;
      srec[u][4 * v + 2] = val.z;
      srec[u][4 * v + 3] = val.w;
    }
  }
  __syncthreads();
  const int g8 = tid & 7, rsub = tid >> 3;
#pragma unroll 1
  for (int i = 0; i < MT_ROWS / 32; ++i) {
    const int32_t r = r0 + rsub + 32 * i;
    if (r >= npad) break;
    uint32_t hv[4] = {0, 0, 0, 0}, lv[4] = {0, 0, 0, 0};
    if (r < nrows) {
      const int32_t sidx = rows[r];
      const int32_t b = (sidx >> 2) - base, sh = (3 - (sidx & 3)) * 2;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int uu = g8 * 8 + u;
        uint32_t byte;
        if (fast)
          byte = (srec[uu][b >> 2] >> ((b & 3) * 8)) & 0xFFu;
        else
          byte = srecoff[uu] >= 0 ? __ldg(geno + srecoff[uu] + (sidx >> 2)) : 0xFFu;
        const uint32_t pair = stab[uu][(byte >> sh) & 3u];
        hv[u >> 1] |= (pair & 0xFFFFu) << ((u & 1) * 16);
        lv[u >> 1] |= (pair >> 16) << ((u & 1) * 16);
      }
    }
    const int64_t off = (int64_t)r * kc + (int64_t)kt * MT_SNP + g8 * 8;
    *(uint4 *)(xhi + off) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
    *(uint4 *)(xlo + off) = make_uint4(lv[0], lv[1], lv[2], lv[3]);
  }
}

/* ------------------------------------------------------------------------------------ */

static PFN_cuTensorMapEncodeTiled_v12000 get_encode(gp_ctx *ctx)
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

/* number of tile pairs of tri_pair for nt tile rows */
static int32_t gram_npairs(int32_t nt)
{
  const int32_t ng = (nt + GRAM_GROUP - 1) / GRAM_GROUP;
  int32_t total = 0;
  for (int32_t gi = 0; gi < ng; ++gi) {
    const int32_t r0 = gi * GRAM_GROUP, nr = (nt < r0 + GRAM_GROUP ? nt : r0 + GRAM_GROUP) - r0;
    for (int32_t gj = 0; gj <= gi; ++gj) {
      const int32_t c0 = gj * GRAM_GROUP, nc = (nt < c0 + GRAM_GROUP ? nt : c0 + GRAM_GROUP) - c0;
      for (int32_t lr = 0; lr < nr; ++lr) total += ((gi == gj ? lr + 1 : nc) + 1) / 2;
    }
  }
  return total;
}

static int make_map(gp_ctx *ctx, CUtensorMap *m, void *base, int32_t rows, int32_t cols,
                    CUtensorMapDataType dt)
{
  PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode(ctx);
  if (!enc) return GP_ERR_CUDA;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {BK, BT};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, dt, 2, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return gp_fail(ctx, GP_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GP_OK;
}

/* FP32 accumulation depth in k-blocks of 64 SNPs before the (hi, lo) add; split budget in bytes */
#define GP_BF16_CHUNK_KB 2
#define GP_BF16_BUDGET (24ll << 30)

int gp_gram_split(gp_ctx *ctx, int precision)
{
  const int fp16 = precision == GP_PREC_SPLIT_FP16;
  const int nmma = precision == GP_PREC_SPLIT_BF16X4 ? 4 : 3;
  const int32_t n = ctx->nrows, nk = ctx->nkept;
  const int32_t npad = (n + BT - 1) / BT * BT;
  const int32_t nt = npad / BT, ntiles = nt * (nt + 1) / 2;
  GP_CUDA(ctx, cudaMemsetAsync(ctx->d_xtx, 0, sizeof(double) * (size_t)n * n, ctx->stream));
  if (nk == 0) return GP_OK;
  const int32_t kpad = (nk + BK - 1) / BK * BK;
  /* super-chunk of kept SNPs so that Xhi + Xlo fit the budget; the budget and the FP32
   * chunk depth can be overridden (GP_BF16_BUDGET_BYTES, GP_BF16_CHUNK_SNPS) for tests and
   * accuracy sweeps */
  int64_t budget = GP_BF16_BUDGET;
  int32_t chunk_kb = GP_BF16_CHUNK_KB;
  {
    const char *e = getenv("GP_BF16_BUDGET_BYTES");
    if (e && atoll(e) > 0) budget = atoll(e);
    e = getenv("GP_BF16_CHUNK_SNPS");
    if (e && atoi(e) >= BK) chunk_kb = atoi(e) / BK;
  }
  int64_t per_col = (int64_t)npad * 4;
  int64_t kc_max = budget / per_col / BK * BK;
  if (kc_max < BK) kc_max = BK;
  int32_t kc = (int32_t)(kpad < kc_max ? kpad : kc_max);
  size_t xbytes = (size_t)npad * kc * 2;
  size_t tab_bytes = (size_t)nk * 16 + 256;
  const int grid0 = ctx->num_sms < ntiles ? ctx->num_sms : ntiles;
  const size_t nsync = (size_t)((kc / BK + GRAM_SYNC_KB - 1) / GRAM_SYNC_KB);
  /* lockstep counters for the waves of either kernel (at least one cluster of two) */
  const size_t waves = (size_t)((ntiles + grid0 - 1) / grid0) > (size_t)gram_npairs(nt)
                           ? (size_t)((ntiles + grid0 - 1) / grid0)
                           : (size_t)gram_npairs(nt);
  const size_t sync_bytes = sizeof(unsigned) * nsync * waves;
  uint8_t *base;
  int rc = gp_scratch2(ctx, 2 * xbytes + tab_bytes + sync_bytes + 512, (void **)&base);
  if (rc) return rc;
  __nv_bfloat16 *xhi = (__nv_bfloat16 *)base;
  __nv_bfloat16 *xlo = (__nv_bfloat16 *)(base + xbytes);
  uint32_t *split = (uint32_t *)(base + 2 * xbytes);
  unsigned *sync_ctr = (unsigned *)(base + ((2 * xbytes + tab_bytes + 255) / 256) * 256);
  int *d_err = ctx->d_err;
  GP_CUDA(ctx, cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  {
    int blocks = (nk + 255) / 256;
    if (blocks > ctx->num_sms * 8) blocks = ctx->num_sms * 8;
    if (fp16)
      k_split_tables<1><<<blocks, 256, 0, ctx->stream>>>(ctx->d_kept, nk, ctx->d_vtab, split);
    else
      k_split_tables<0><<<blocks, 256, 0, ctx->stream>>>(ctx->d_kept, nk, ctx->d_vtab, split);
    GP_LAUNCH_CHECK(ctx, "k_split_tables");
  }
  typedef void (*gram_kern_t)(const CUtensorMap, const CUtensorMap, int32_t, int32_t, int32_t,
                              int32_t, double *, int32_t, int32_t, unsigned *, int *);
  gram_kern_t kern = fp16 ? k_gram_split<1, 3, 1>
                          : (nmma == 4 ? k_gram_split<0, 4, 1> : k_gram_split<0, 3, 1>);
  gram_kern_t kern2 = fp16 ? k_gram_split<1, 3, 2>
                           : (nmma == 4 ? k_gram_split<0, 4, 2> : k_gram_split<0, 3, 2>);
  gram_kern_t kern4 = fp16 ? k_gram_split<1, 3, 4>
                           : (nmma == 4 ? k_gram_split<0, 4, 4> : k_gram_split<0, 3, 4>);
  /* clusters of four CTAs (2 x 2 tiles sharing row and column boxes), else two (two tiles of
   * a row sharing its boxes), else one CTA per tile; GP_GRAM_CLUSTER=1|2|4 caps the size.
   * The next smaller size is used when the cluster launch is refused. */
  int cl = ctx->gram_cluster_cap > 0 ? ctx->gram_cluster_cap : 4;
  {
    const char *ce = getenv("GP_GRAM_CLUSTER");
    if (ce && atoi(ce) >= 1 && atoi(ce) < cl) cl = atoi(ce) >= 4 ? 4 : (atoi(ce) >= 2 ? 2 : 1);
  }
  const int32_t nq = (nt + 1) / 2;
  const int32_t nwork_cl[5] = {0, ntiles, gram_npairs(nt), 0, nq * (nq + 1) / 2};
  int32_t ncl = 0;
  for (; cl > 1; cl /= 2) {
    gram_kern_t kc = cl == 4 ? kern4 : kern2;
    GP_CUDA(ctx, cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, GRAM_SMEM));
    cudaLaunchConfig_t qc = {};
    qc.gridDim = dim3((unsigned)((ctx->num_sms / cl) * cl));
    qc.blockDim = dim3(GRAM_THREADS);
    qc.dynamicSmemBytes = GRAM_SMEM;
    cudaLaunchAttribute qa[1];
    qa[0].id = cudaLaunchAttributeClusterDimension;
    qa[0].val.clusterDim.x = (unsigned)cl;
    qa[0].val.clusterDim.y = 1;
    qa[0].val.clusterDim.z = 1;
    qc.attrs = qa;
    qc.numAttrs = 1;
    int maxcl = 0;
    if (cudaOccupancyMaxActiveClusters(&maxcl, (const void *)kc, &qc) != cudaSuccess) {
      cudaGetLastError();
      maxcl = 0;
    }
    ncl = maxcl < ctx->num_sms / cl ? maxcl : ctx->num_sms / cl;
    if (ncl > nwork_cl[cl]) ncl = nwork_cl[cl];
    if (ncl >= 1) break;
  }
  if (cl < 2) ncl = 0;
  GP_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, GRAM_SMEM));
  CUtensorMap mhi, mlo;
  CUtensorMapDataType dt = fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  rc = make_map(ctx, &mhi, xhi, npad, kc, dt);
  if (!rc) rc = make_map(ctx, &mlo, xlo, npad, kc, dt);
  if (rc) return rc;
  int grid = grid0;
  for (int32_t k0 = 0; k0 < kpad; k0 += kc) {
    int32_t kcur = kpad - k0 < kc ? kpad - k0 : kc;
    /* columns beyond kcur in this super-chunk are zero (k >= nkept guard covers the tail) */
    dim3 tgrid((unsigned)(kc / MT_SNP), (unsigned)((npad + MT_ROWS - 1) / MT_ROWS));
    k_split_transpose<<<tgrid, 256, 0, ctx->stream>>>(ctx->d_geno, ctx->rlen_dev, ctx->d_rows, n,
                                                      ctx->d_cols, ctx->d_kept, nk, split, k0, kc,
                                                      npad, xhi, xlo);
    GP_LAUNCH_CHECK(ctx, "k_split_transpose");
    int32_t nkb = kcur / BK;
    GP_CUDA(ctx, cudaMemsetAsync(sync_ctr, 0, sync_bytes, ctx->stream));
    /* cooperative launch: the producers' lockstep points need every CTA resident */
    int32_t a_nt = ntiles, a_rows = nt, a_nkb = nkb, a_ck = chunk_kb, a_n = n,
            a_acc = k0 > 0 ? 1 : 0;
    double *a_xtx = ctx->d_xtx;
    bool launched = false;
    while (!launched && ncl > 0) {
      cudaLaunchConfig_t lc = {};
      lc.gridDim = dim3((unsigned)(cl * ncl));
      lc.blockDim = dim3(GRAM_THREADS);
      lc.dynamicSmemBytes = GRAM_SMEM;
      lc.stream = ctx->stream;
      cudaLaunchAttribute la[2];
      la[0].id = cudaLaunchAttributeClusterDimension;
      la[0].val.clusterDim.x = (unsigned)cl;
      la[0].val.clusterDim.y = 1;
      la[0].val.clusterDim.z = 1;
      la[1].id = cudaLaunchAttributeCooperative;
      la[1].val.cooperative = 1;
      lc.attrs = la;
      lc.numAttrs = 2;
      cudaError_t le = cudaLaunchKernelEx(&lc, cl == 4 ? kern4 : kern2, mhi, mlo, nwork_cl[cl],
                                          a_rows, a_nkb, a_ck, a_xtx, a_n, a_acc, sync_ctr, d_err);
      if (le == cudaSuccess) {
        launched = true;
      } else {
        cudaGetLastError();
        /* refused: the next smaller cluster (same count of SMs), finally one CTA per tile */
        cl /= 2;
        ncl = cl > 1 ? ((ctx->num_sms / cl) < nwork_cl[cl] ? ctx->num_sms / cl : nwork_cl[cl]) : 0;
      }
    }
    if (!launched) {
      void *args[] = {&mhi, &mlo, &a_nt, &a_rows, &a_nkb, &a_ck, &a_xtx, &a_n, &a_acc, &sync_ctr,
                      &d_err};
      GP_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(GRAM_THREADS),
                                               args, GRAM_SMEM, ctx->stream));
    }
    ctx->launches++;
    ctx->gram_launches++;
  }
  int herr = 0;
  GP_CUDA(ctx, gp_memcpy(ctx, &herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (herr == GP_KERR_CLUSTER) {
    /* the launch ran without its clusters (every CTA refused before any load or MMA, so
     * nothing was written): redo the whole Gram on the one-CTA schedule, which needs no
     * cluster, and keep that schedule for this handle */
    if (ctx->gram_cluster_cap == 1)
      return gp_fail(ctx, GP_ERR_CUDA, "split Gram: the cluster launch was not honoured");
    ctx->gram_cluster_cap = 1;
    return gp_gram_split(ctx, precision);
  }
  if (herr) return gp_fail(ctx, GP_ERR_TIMEOUT, "split-BF16 Gram kernel wait timed out (code %d)", herr);
  return GP_OK;
}
