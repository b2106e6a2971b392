/*
 * Blackwell (sm_103a) primitives used by the tensor-core kernels, as inline PTX:
 * mbarriers with bounded waits, TMA 2-D tile loads, TMEM allocation, tcgen05.mma (kind::f16,
 * cta_group::1), tcgen05.commit, tcgen05.ld / tcgen05.st and the UMMA shared-memory and
 * instruction descriptors for K-major operands in the 128-byte swizzled layout.
 *
 * Every wait is bounded by wall time (%globaltimer): when it runs out the kernel records an
 * error code in global memory, raises a shared abort flag so that the other warps stop
 * waiting, and unwinds; the host turns the code into GP_ERR_TIMEOUT.
 */
#ifndef GP_TC_CUH
#define GP_TC_CUH

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#define GP_WAIT_NS (2000000000ull) /* 2 s per wait */

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

/* ---- mbarrier ------------------------------------------------------------------------ */

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t *bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok;
}

/*
 * Wait until the phase of `bar` with the given parity has completed.  Returns false when
 * the shared abort flag is raised or the wait runs past GP_WAIT_NS (then raises the flag
 * and records `code` in *err).
 */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          int *err, int code)
{
  if (mbar_try_wait(bar, parity)) return true;
  uint64_t t0 = globaltimer_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer_ns() - t0 > GP_WAIT_NS) {
      *abort_flag = 1;
      atomicCAS(err, 0, code);
      return false;
    }
  }
}

/* ---- TMA ---------------------------------------------------------------------------- */

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int32_t x, int32_t y)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

/* the same box into the same shared-memory offset of every CTA of the cluster in cta_mask,
 * completing bytes on the mbarrier at the same offset in each */
__device__ __forceinline__ void tma_load_2d_mc(void *dst, const CUtensorMap *map, uint64_t *bar,
                                               int32_t x, int32_t y, uint16_t cta_mask)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar)), "h"(cta_mask)
      : "memory");
}

__device__ __forceinline__ uint32_t cluster_ctarank()
{
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id_x()
{
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_nctarank()
{
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count_x()
{
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
/* every thread of every CTA of the cluster (release / acquire) */
__device__ __forceinline__ void cluster_sync_all()
{
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
               ::: "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap *map)
{
  asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

/* ---- TMEM ---------------------------------------------------------------------------- */

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

/* 32 lanes x 16 consecutive 32-bit columns: thread t gets lane (base+t), columns c..c+15 */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r)
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t *r)
{
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

/* ---- UMMA -------------------------------------------------------------------------- */

/*
 * Shared-memory matrix descriptor (sm_100 family) for a K-major operand tile whose rows are
 * 128 bytes (64 bf16) written by TMA with the 128-byte swizzle: 8-row groups of 1024 bytes
 * (stride byte offset), start address in 16-byte units, descriptor version 1, layout type 2
 * (SWIZZLE_128B).  The leading byte offset is unused for this layout (the MMA's K extent of
 * 32 bytes stays inside one swizzled row).
 */
__device__ __forceinline__ uint64_t sdesc_k128(uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1u << 16;            /* LBO = 16 bytes (unused) */
  d |= (uint64_t)(1024u >> 4) << 32;  /* SBO = 1024 bytes */
  d |= (uint64_t)1u << 46;            /* version */
  d |= (uint64_t)2u << 61;            /* SWIZZLE_128B */
  return d;
}

/* instruction descriptor: kind::f16, A = B = BF16, D = F32, both K-major, M x N */
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t M, uint32_t N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

/* instruction descriptor: kind::f16, A = B = F16, D = F32, both K-major, M x N */
__host__ __device__ constexpr uint32_t idesc_f16_f32(uint32_t M, uint32_t N)
{
  return (1u << 4) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

/* one tcgen05.mma kind::f16 (bf16 or f16 operands, as the instruction descriptor says) */
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
/* the commit's arrive on the mbarrier at bar's offset in every CTA of cta_mask */
__device__ __forceinline__ void umma_commit_mc(uint64_t *bar, uint16_t cta_mask)
{
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(smem_u32(bar)), "h"(cta_mask)
      : "memory");
}

#endif
