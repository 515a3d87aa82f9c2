/*
 * Fused evaluation of the surrogate network on sm_103a: one persistent
 * kernel per batch of pairs, 128 pairs (rows) per tile, 8 warps per CTA,
 * one CTA per SM.
 *
 *   layer 1 (3 -> 256)    CUDA cores, FP32, SiLU, written as BF16 straight
 *                         into the shared-memory A tile (K-major core
 *                         matrices, 64 KB)
 *   layers 2, 3 (256^2)   tensor cores: tcgen05.mma M = 128, N = 64 per
 *                         weight chunk, K = 256, FP32 accumulator in tensor
 *                         memory (256 columns); the weights stream from the
 *                         pre-laid-out weight image (L2-resident, 8 chunks of
 *                         32 KB) into a ring of four shared-memory buffers by
 *                         bulk TMA copies issued up to four chunks ahead, so the
 *                         next layer's weights land during an epilogue; the epilogue (bias,
 *                         SiLU, BF16) reads the accumulator with tcgen05.ld
 *                         and writes the next layer's A tile in place
 *   layer 4 (256 -> 48)   tensor cores, N = 48, W4 resident in shared memory;
 *                         bias and FP32 rows to global memory
 *
 * The activations never leave the SM: per pair the kernel reads 16 bytes of
 * features and writes 192 bytes of outputs; the weights (280 KB) are re-read
 * from L2 once per tile.  One thread issues every MMA and bulk copy; every
 * wait on an mbarrier is bounded, and a wait that runs out sets *err and
 * sends the CTA to its clean-up, which waits (bounded) for the copies and
 * MMAs it has in flight before freeing its tensor memory.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kqed_internal.h"
#include "kqed_mlp.h"
#include "kqed_umma.h"

namespace kqed {
namespace mlp {

using namespace umma;

constexpr int kIThreads = 256;
constexpr int kIA = 128 * kH * 2;                 /* A tile, 64 KB */
constexpr int kIParams = kH * 3 + kH + kH + kH + kNop;   /* W1 b1 b2 b3 b4 */
constexpr int kWBufs = 4;                         /* weight-chunk ring in shared memory */
constexpr int kInferSmem =
    kIA + kWBufs * (int)kWimgChunk + (int)kWimgW4 + kIParams * 4 + 1024;

__device__ __forceinline__ float silu_i(float z) { return z / (1.0f + __expf(-z)); }

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}

/* the weight image from the fp32 parameters */
__global__ void build_wimg_kernel(const float *P, __nv_bfloat16 *wimg)
{
  const size_t n23 = (size_t)8 * 64 * kH, n4 = (size_t)kNop * kH;
  unsigned char *img = reinterpret_cast<unsigned char *>(wimg);
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n23 + n4;
       e += (size_t)gridDim.x * blockDim.x) {
    if (e < n23) {
      const int chunk = (int)(e / (64 * kH));            /* 0..3 W2, 4..7 W3 */
      const int rem = (int)(e % (64 * kH));
      const int nl = rem / kH, k = rem % kH;
      const int n = 64 * (chunk & 3) + nl;
      const float v = P[(chunk < 4 ? kOW2 : kOW3) + (size_t)n * kH + k];
      *reinterpret_cast<__nv_bfloat16 *>(img + chunk * kWimgChunk + kmajor_off(nl, k, 64)) =
          __float2bfloat16_rn(v);
    } else {
      const int q = (int)(e - n23);
      const int n = q / kH, k = q % kH;
      const float v = n < kNo ? P[kOW4 + (size_t)n * kH + k] : 0.0f;
      *reinterpret_cast<__nv_bfloat16 *>(img + 8 * kWimgChunk + kmajor_off(n, k, kNop)) =
          __float2bfloat16_rn(v);
    }
  }
}

__global__ void __launch_bounds__(kIThreads, 1) mlp_infer_kernel(InferArgs a)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char *sA = base;
  unsigned char *sW[kWBufs];
  for (int i = 0; i < kWBufs; i++) sW[i] = base + kIA + i * kWimgChunk;
  unsigned char *sW4 = base + kIA + kWBufs * kWimgChunk;
  float *sP = reinterpret_cast<float *>(sW4 + kWimgW4);
  float *sW1 = sP, *sb1 = sP + 3 * kH, *sb2 = sb1 + kH, *sb3 = sb2 + kH, *sb4 = sb3 + kH;
  __shared__ uint64_t wbar[kWBufs], w4bar, ldone, mdone[kWBufs];
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail;

  const size_t n = a.count ? min(a.rows, (size_t)*a.count) : a.rows;
  const size_t ntiles = (n + 127) / 128;
  if ((size_t)blockIdx.x >= ntiles) return;
  const size_t my_tiles = (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x;
  const size_t total_chunks = 8 * my_tiles;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned char *img = reinterpret_cast<const unsigned char *>(a.wimg);

  if (tid == 0) {
    for (int i = 0; i < kWBufs; i++) {
      mbar_init(&wbar[i], 1);
      mbar_init(&mdone[i], 1);
    }
    mbar_init(&w4bar, 1);
    mbar_init(&ldone, 1);
    fence_mbar_init();
    s_fail = 0;
  }
  if (warp == 0) {
    tmem_alloc(&s_taddr, 256);
    tmem_relinquish();
  }
  for (int i = tid; i < 3 * kH; i += kIThreads) sW1[i] = a.P[kOW1 + i];
  for (int i = tid; i < kH; i += kIThreads) {
    sb1[i] = a.P[kOB1 + i];
    sb2[i] = a.P[kOB2 + i];
    sb3[i] = a.P[kOB3 + i];
  }
  if (tid < kNop) sb4[tid] = a.P[kOB4 + tid];
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_taddr;

  size_t loads = 0;      /* weight chunks whose bulk copy was issued */
  size_t g = 0;          /* weight chunks consumed */
  uint32_t lphase = 0;   /* completed phases of ldone */
  if (tid == 0) {
    mbar_expect_tx(&w4bar, (uint32_t)kWimgW4);
    bulk_g2s(sW4, img + 8 * kWimgChunk, (uint32_t)kWimgW4, &w4bar);
    for (int c = 0; c < kWBufs; c++) {
      mbar_expect_tx(&wbar[c], (uint32_t)kWimgChunk);
      bulk_g2s(sW[c], img + c * kWimgChunk, (uint32_t)kWimgChunk, &wbar[c]);
    }
  }
  loads = kWBufs;   /* total_chunks >= 8 >= kWBufs */
  bool w4_ready = false;
  const uint32_t a0 = smem_u32(sA);

  for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const size_t row0 = tile * 128;
    /* ---- layer 1: thread -> (row, half of the 256 outputs) */
    {
      const int r = tid & 127, h = tid >> 7;
      const size_t row = row0 + r;
      const float4 f = row < n ? a.feat[row] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll 2
      for (int c = 0; c < 16; c++) {
        const int j0 = 128 * h + 8 * c;
        float z[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const int j = j0 + i;
          z[i] = silu_i(fmaf(sW1[3 * j + 2], f.z, fmaf(sW1[3 * j + 1], f.y,
                                                         fmaf(sW1[3 * j], f.x, sb1[j]))));
        }
        uint4 v;
        v.x = pack_bf16(z[0], z[1]);
        v.y = pack_bf16(z[2], z[3]);
        v.z = pack_bf16(z[4], z[5]);
        v.w = pack_bf16(z[6], z[7]);
        *reinterpret_cast<uint4 *>(sA + kmajor_off(r, j0, 128)) = v;
      }
    }
    fence_proxy_async();
    __syncthreads();

    /* ---- layers 2 and 3 */
    for (int l = 0; l < 2; l++) {
      if (tid == 0) {
        fence_after_sync();
        for (int q = 0; q < 4 && !s_fail; q++) {
          const int b = (int)(g % kWBufs);
          if (!mbar_wait(&wbar[b], (uint32_t)((g / kWBufs) & 1))) { s_fail = 1; break; }
          const uint32_t b0 = smem_u32(sW[b]);
#pragma unroll
          for (int kk = 0; kk < kH / 16; kk++)
            mma_bf16(tmem + 64 * q, sdesc(a0 + kk * 2 * (128 * 16), 128 * 16, 128),
                     sdesc(b0 + kk * 2 * (64 * 16), 64 * 16, 128), idesc_bf16(128, 64),
                     kk > 0 ? 1u : 0u);
          mma_commit(&mdone[b]);
          if (g >= 1) {
            /* the MMAs of chunk g - 1 are done with their buffer: refill it
               with chunk g - 1 + kWBufs, kWBufs - 1 chunks ahead */
            if (!mbar_wait(&mdone[(g - 1) % kWBufs], (uint32_t)(((g - 1) / kWBufs) & 1))) {
              s_fail = 1;
              g++;
              break;
            }
            const size_t c = g - 1 + kWBufs;
            if (c < total_chunks) {
              const int cb = (int)(c % kWBufs);
              mbar_expect_tx(&wbar[cb], (uint32_t)kWimgChunk);
              bulk_g2s(sW[cb], img + (c & 7) * kWimgChunk, (uint32_t)kWimgChunk, &wbar[cb]);
              loads = c + 1;
            }
          }
          g++;
        }
        if (!s_fail) mma_commit(&ldone);
      }
      __syncthreads();
      if (s_fail) break;
      if (!mbar_wait(&ldone, lphase & 1)) s_fail = 1;
      lphase++;
      __syncthreads();
      if (s_fail) break;
      fence_after_sync();
      /* epilogue: warp -> (32 rows, half of the columns) */
      {
        const int rq = warp & 3, ch = warp >> 2;
        const int r = 32 * rq + lane;
        const float *bias = l == 0 ? sb2 : sb3;
        const uint32_t trow = tmem + ((uint32_t)(32 * rq) << 16);
        for (int c0 = 128 * ch; c0 < 128 * ch + 128; c0 += 16) {
          float v[16];
          tmem_ld16(trow + (uint32_t)c0, v);
          uint4 lo, hi;
          lo.x = pack_bf16(silu_i(v[0] + bias[c0 + 0]), silu_i(v[1] + bias[c0 + 1]));
          lo.y = pack_bf16(silu_i(v[2] + bias[c0 + 2]), silu_i(v[3] + bias[c0 + 3]));
          lo.z = pack_bf16(silu_i(v[4] + bias[c0 + 4]), silu_i(v[5] + bias[c0 + 5]));
          lo.w = pack_bf16(silu_i(v[6] + bias[c0 + 6]), silu_i(v[7] + bias[c0 + 7]));
          hi.x = pack_bf16(silu_i(v[8] + bias[c0 + 8]), silu_i(v[9] + bias[c0 + 9]));
          hi.y = pack_bf16(silu_i(v[10] + bias[c0 + 10]), silu_i(v[11] + bias[c0 + 11]));
          hi.z = pack_bf16(silu_i(v[12] + bias[c0 + 12]), silu_i(v[13] + bias[c0 + 13]));
          hi.w = pack_bf16(silu_i(v[14] + bias[c0 + 14]), silu_i(v[15] + bias[c0 + 15]));
          *reinterpret_cast<uint4 *>(sA + kmajor_off(r, c0, 128)) = lo;
          *reinterpret_cast<uint4 *>(sA + kmajor_off(r, c0 + 8, 128)) = hi;
        }
      }
      fence_before_sync();
      fence_proxy_async();
      __syncthreads();
    }
    if (s_fail) break;

    /* ---- layer 4 */
    if (tid == 0) {
      if (!w4_ready) {
        if (!mbar_wait(&w4bar, 0)) s_fail = 1;
        w4_ready = true;
      }
      if (!s_fail) {
        fence_after_sync();
        const uint32_t b0 = smem_u32(sW4);
#pragma unroll
        for (int kk = 0; kk < kH / 16; kk++)
          mma_bf16(tmem, sdesc(a0 + kk * 2 * (128 * 16), 128 * 16, 128),
                   sdesc(b0 + kk * 2 * (kNop * 16), kNop * 16, 128), idesc_bf16(128, kNop),
                   kk > 0 ? 1u : 0u);
        mma_commit(&ldone);
      }
    }
    __syncthreads();
    if (s_fail) break;
    if (!mbar_wait(&ldone, lphase & 1)) s_fail = 1;
    lphase++;
    __syncthreads();
    if (s_fail) break;
    fence_after_sync();
    if (warp < 4) {
      const int r = 32 * warp + lane;
      const size_t row = row0 + r;
      const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
      for (int c0 = 0; c0 < kNop; c0 += 16) {
        float v[16];
        tmem_ld16(trow + (uint32_t)c0, v);
        if (row < n) {
          float4 *o = reinterpret_cast<float4 *>(a.Y + row * kNop + c0);
#pragma unroll
          for (int i = 0; i < 4; i++)
            o[i] = make_float4(v[4 * i] + sb4[c0 + 4 * i], v[4 * i + 1] + sb4[c0 + 4 * i + 1],
                               v[4 * i + 2] + sb4[c0 + 4 * i + 2],
                               v[4 * i + 3] + sb4[c0 + 4 * i + 3]);
        }
      }
    }
    fence_before_sync();
    __syncthreads();
  }

  /* clean-up: bulk copies still in flight (weight chunks issued but not
     consumed, W4 if never waited for) and, after a failure, the MMAs */
  if (tid == 0) {
    if (s_fail && a.err) atomicExch(a.err, 1);
    for (size_t c = g; c < loads; c++)
      mbar_wait(&wbar[c % kWBufs], (uint32_t)((c / kWBufs) & 1), 1u << 26);
    if (!w4_ready) mbar_wait(&w4bar, 0, 1u << 26);
    if (s_fail) {
      mma_commit(&ldone);
      mbar_wait(&ldone, lphase & 1, 1u << 26);
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

cudaError_t launch_build_wimg(const float *P, __nv_bfloat16 *wimg, cudaStream_t s)
{
  build_wimg_kernel<<<256, 256, 0, s>>>(P, wimg);
  g_launches++;
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const InferArgs &a, cudaStream_t s)
{
  if (a.rows == 0) return cudaSuccess;
  cudaError_t e =
      cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;
  const size_t tiles = (a.rows + 127) / 128;
  const unsigned grid = (unsigned)(tiles < (size_t)sms ? tiles : (size_t)sms);
  mlp_infer_kernel<<<grid, kIThreads, kInferSmem, s>>>(a);
  g_launches++;
  return cudaGetLastError();
}

} // namespace mlp
} // namespace kqed
