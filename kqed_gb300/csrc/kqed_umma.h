/*
 * Blackwell (sm_103a) tensor-core helpers: tcgen05 MMA with the accumulator
 * in tensor memory (TMEM), shared-memory matrix descriptors, mbarrier waits.
 * Inline PTX only; used by the surrogate's BF16 GEMMs (kqed_mlp_gemm.cu).
 *
 * Operand layout.  Every operand is staged K-major without swizzling, in
 * 8-row x 16-byte "core matrices" (8 rows of 8 bf16, 128 contiguous bytes).
 * For a tile of R rows (R = M for A, N for B) and 64 K elements the core
 * matrix (row group g, K chunk c) sits at byte ((c * R / 8) + g) * 128, row r
 * of it at +16 r.  In the descriptor the leading-dimension byte offset is
 * then the K-direction stride between core matrices, R * 16 bytes, and the
 * stride-dimension byte offset the row-group stride, 128 bytes; one MMA
 * consumes K = 16, i.e. two K chunks, and the next MMA's descriptor starts
 * 2 * R * 16 bytes further.
 *
 * Waits are bounded: a wait that runs out of iterations returns false and the
 * caller records an error status instead of spinning forever.
 */
#ifndef KQED_UMMA_H
#define KQED_UMMA_H

#include <cuda_bf16.h>
#include <stdint.h>

namespace kqed {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

/* shared-memory matrix descriptor, no swizzle (layout type 0), descriptor
   version 1 (bits 46-47), base offset 0, relative leading-dimension mode */
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

/* instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32
   accumulator, dense, M x N */
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync()
{
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync()
{
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
/* generic-proxy shared-memory writes made visible to the tensor cores */
__device__ __forceinline__ void fence_proxy_async()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
/* bounded wait for the phase with the given parity to complete; false when
   the limit ran out */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit = 1u << 22)
{
  for (uint32_t i = 0; i < limit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

/* bulk (TMA) copy global -> shared of `bytes` (a multiple of 16, both
   addresses 16-byte aligned), completing on the mbarrier as transaction
   bytes; the issuing thread first announces the bytes with expect_tx */
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst_smem, const void *src, uint32_t bytes,
                                         uint64_t *bar)
{
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst_smem)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

/* D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread */
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
/* arrive on the mbarrier once every MMA issued so far by this thread is done */
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

/* 16 consecutive FP32 columns of this thread's TMEM lane (warp w of the
   warpgroup reads lanes 32 w .. 32 w + 31) */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

/* byte offset of element (row, k) in a K-major no-swizzle tile of R rows */
__host__ __device__ __forceinline__ uint32_t kmajor_off(int row, int k, int R)
{
  return (uint32_t)((((k >> 3) * (R >> 3)) + (row >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

} // namespace umma
} // namespace kqed

#endif
