/*
 * BF16 GEMM on the sm_103a tensor cores (tcgen05.mma, FP32 accumulator in
 * tensor memory) for the learned weight-function surrogate: its training
 * (forward, both backward products, weight gradients) and its layer-wise
 * evaluation run through this one kernel.
 *
 *   C[m][n] = epilogue( sum_k A(m, k) B(n, k) ),  A, B bf16, C fp32 / bf16
 *
 * A(m, k) = A[m * sAm + k * sAk] and B(n, k) = B[n * sBn + k * sBk]: any
 * strides, so X W^T, dZ W and dZ^T H (transposed operands) are the same
 * kernel.  A CTA of 128 threads owns a 128 x BN tile (BN <= 256, multiple of
 * 16) with the accumulator in TMEM; K runs in stages of 64 through two
 * shared-memory buffers, the next stage being staged by all threads while
 * the tensor cores work on the current one.  blockIdx.z splits K: split z
 * covers k in [z * ksplit, (z + 1) * ksplit) and writes its own partial
 * product (mode STORE), so weight gradients over large batches reduce in a
 * fixed order afterwards.
 *
 * Epilogue modes (the layer structure of the surrogate MLP):
 *   STORE   cf[z * pstride + m * ldc + n] = acc
 *   HIDDEN  z = acc + bias[n]; cf[m ldc + n] = z; cb[m ldb + n] = bf16(silu(z))
 *   OUT     cf[m ldc + n] = acc + bias[n]
 *   BWD     d = acc * silu'(zin[m ldc + n]); cb[m ldb + n] = bf16(d); cf[...] = d if cf
 *
 * Every mbarrier wait is bounded; a wait that runs out sets *err and the
 * CTA skips to its clean-up, which waits (again bounded) for its MMAs in
 * flight before freeing its tensor memory.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "kqed_internal.h"
#include "kqed_mlp.h"
#include "kqed_umma.h"

namespace kqed {
namespace mlp {

using namespace umma;

constexpr int kBM = 128;
constexpr int kBK = 64;
constexpr int kMaxBN = 256;
constexpr int kStageA = kBM * kBK * 2;        /* 16 KB */
constexpr int kStageB = kMaxBN * kBK * 2;     /* 32 KB */
constexpr int kGemmSmem = 2 * (kStageA + kStageB) + 1024;

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_(float z) { return z * sigmoidf_(z); }
__device__ __forceinline__ float dsilu_(float z)
{
  const float s = sigmoidf_(z);
  return s * (1.0f + z * (1.0f - s));
}

/* stage rows [r0, r0 + R) x k in [k0, k0 + 64) of a strided bf16 operand into
   the K-major core-matrix layout (zero outside [0, rows) x [0, kend)) */
__device__ __forceinline__ void stage_operand(unsigned char *dst, int R, const __nv_bfloat16 *src,
                                              long long sr, long long sk, int r0, int rows, int k0,
                                              int kend)
{
  const int chunks = R * (kBK / 8);
  const bool krow = (sk == 1);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    int r, kc;
    if (krow) { r = c / (kBK / 8); kc = c % (kBK / 8); }   /* a row's chunks on adjacent threads */
    else { r = c % R; kc = c / R; }                        /* adjacent rows on adjacent threads */
    const int gr = r0 + r, gk = k0 + kc * 8;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (gr < rows && gk < kend) {
      const __nv_bfloat16 *p = src + (long long)gr * sr + (long long)gk * sk;
      if (krow && gk + 8 <= kend && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
        v = __ldg(reinterpret_cast<const uint4 *>(p));
      } else {
        unsigned short e[8];
#pragma unroll
        for (int i = 0; i < 8; i++)
          e[i] = (gk + i < kend) ? __bfloat16_as_ushort(p[(long long)i * sk]) : (unsigned short)0;
        v.x = e[0] | ((unsigned)e[1] << 16);
        v.y = e[2] | ((unsigned)e[3] << 16);
        v.z = e[4] | ((unsigned)e[5] << 16);
        v.w = e[6] | ((unsigned)e[7] << 16);
      }
    }
    *reinterpret_cast<uint4 *>(dst + kmajor_off(r, kc * 8, R)) = v;
  }
}

__global__ void __launch_bounds__(128) gemm_kernel(GemmArgs g)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char *sa[2] = {base, base + kStageA};
  unsigned char *sb[2] = {base + 2 * kStageA, base + 2 * kStageA + kStageB};
  __shared__ uint64_t bar[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail;

  const int BN = g.bn;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  if (g.Mdev) {
    /* rows counted on the device: tiles beyond them have nothing to do */
    const int mr = (int)min((unsigned)g.M, *g.Mdev);
    if (m0 >= mr) return;
    g.M = mr;
  }
  const int kb = blockIdx.z * g.ksplit;
  const int ke = min(g.K, kb + g.ksplit);
  const int nst = ke > kb ? (ke - kb + kBK - 1) / kBK : 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_fail = 0;
  }
  if (warp == 0) {
    tmem_alloc(&s_taddr, 256);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_taddr;
  const uint32_t idesc = idesc_bf16(kBM, BN);
  const uint32_t lbo_a = kBM * 16, lbo_b = (uint32_t)BN * 16;

  int issued = 0;   /* stages whose MMAs were issued */
  for (int s = 0; s < nst; s++) {
    const int b = s & 1;
    if (s >= 2) {
      /* buffer b was last read by the MMAs of stage s - 2 */
      if (!mbar_wait(&bar[b], ((s - 2) >> 1) & 1)) {
        if (threadIdx.x == 0) s_fail = 1;
      }
    }
    __syncthreads();
    if (s_fail) break;
    const int k0 = kb + s * kBK;
    stage_operand(sa[b], kBM, g.A, g.sAm, g.sAk, m0, g.M, k0, ke);
    stage_operand(sb[b], BN, g.B, g.sBn, g.sBk, n0, g.N, k0, ke);
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      fence_after_sync();
      const uint32_t a0 = smem_u32(sa[b]), b0 = smem_u32(sb[b]);
#pragma unroll
      for (int j = 0; j < kBK / 16; j++)
        mma_bf16(tmem, sdesc(a0 + 2 * j * lbo_a, lbo_a, 128), sdesc(b0 + 2 * j * lbo_b, lbo_b, 128),
                 idesc, (s > 0 || j > 0) ? 1u : 0u);
      mma_commit(&bar[b]);
    }
    issued = s + 1;
  }
  /* all MMAs done: the last commit covers every earlier one */
  if (issued > 0) {
    const int sl = issued - 1;
    if (!mbar_wait(&bar[sl & 1], (sl >> 1) & 1)) {
      if (threadIdx.x == 0) s_fail = 1;
    }
  }
  __syncthreads();
  fence_after_sync();
  if (s_fail) {
    /* give the MMAs in flight a second, longer bounded wait before the
       tensor memory they write is freed */
    if (threadIdx.x == 0) {
      if (g.err) atomicExch(g.err, 1);
      if (issued > 0) mbar_wait(&bar[(issued - 1) & 1], ((issued - 1) >> 1) & 1, 1u << 26);
    }
    __syncthreads();
  } else {
    const int row = m0 + warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      if (nst > 0) tmem_ld16(trow + (uint32_t)c0, v);
      else {
#pragma unroll
        for (int i = 0; i < 16; i++) v[i] = 0.0f;
      }
      if (row >= g.M) continue;
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int n = n0 + c0 + i;
        if (n >= g.N) break;
        const float acc = v[i];
        switch (g.mode) {
        case kStore:
          g.cf[(long long)blockIdx.z * g.pstride + (long long)row * g.ldc + n] = acc;
          break;
        case kHidden: {
          const float z = acc + (g.bias ? g.bias[n] : 0.0f);
          if (g.cf) g.cf[(long long)row * g.ldc + n] = z;
          g.cb[(long long)row * g.ldb + n] = __float2bfloat16_rn(silu_(z));
          break;
        }
        case kOut:
          g.cf[(long long)row * g.ldc + n] = acc + (g.bias ? g.bias[n] : 0.0f);
          break;
        default: { /* kBwd */
          const float d = acc * dsilu_(g.zin[(long long)row * g.ldc + n]);
          if (g.cb) g.cb[(long long)row * g.ldb + n] = __float2bfloat16_rn(d);
          if (g.cf) g.cf[(long long)row * g.ldc + n] = d;
          break;
        }
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

int gemm_smem_bytes() { return kGemmSmem; }

/* one device int per device for the kernels' timeout flag (allocated on
   first use, kept for the life of the process) */
int device_error_flag(int **out)
{
  static std::mutex mu;
  static int *flags[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> g(mu);
  if (!flags[dev] && cudaMalloc(&flags[dev], sizeof(int)) != cudaSuccess) return 1;
  *out = flags[dev];
  return 0;
}

cudaError_t launch_gemm(const GemmArgs &g0, int splits, cudaStream_t s)
{
  GemmArgs g = g0;
  if (g.M <= 0 || g.N <= 0 || g.K < 0 || splits < 1) return cudaErrorInvalidValue;
  g.bn = g.N >= kMaxBN ? kMaxBN : ((g.N + 15) / 16) * 16;
  g.ksplit = (g.K + splits - 1) / splits;
  g.ksplit = ((g.ksplit + kBK - 1) / kBK) * kBK;
  if (g.ksplit == 0) g.ksplit = kBK;
  const cudaError_t e =
      cudaFuncSetAttribute(gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
  if (e != cudaSuccess) return e;
  const dim3 grid((g.M + kBM - 1) / kBM, (g.N + g.bn - 1) / g.bn, splits);
  gemm_kernel<<<grid, 128, kGemmSmem, s>>>(g);
  g_launches++;
  return cudaGetLastError();
}

} // namespace mlp
} // namespace kqed

/* --------------------------------------------------------- C-ABI (test) */

extern "C" int kqed_bf16_gemm(const void *d_a, long long sam, long long sak, const void *d_b,
                              long long sbn, long long sbk, int M, int N, int K, int splits,
                              float *d_c, long long ldc, void *stream)
{
  using namespace kqed::mlp;
  if (!d_a || !d_b || !d_c || M <= 0 || N <= 0 || K < 0 || splits < 1 || ldc < N)
    return kqed::set_error("kqed_bf16_gemm: bad arguments");
  int *err = nullptr;
  if (device_error_flag(&err)) return kqed::set_error("kqed_bf16_gemm: no error flag");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GemmArgs g{};
  g.A = static_cast<const __nv_bfloat16 *>(d_a);
  g.sAm = sam;
  g.sAk = sak;
  g.B = static_cast<const __nv_bfloat16 *>(d_b);
  g.sBn = sbn;
  g.sBk = sbk;
  g.M = M;
  g.N = N;
  g.K = K;
  g.mode = kStore;
  g.cf = d_c;
  g.ldc = ldc;
  g.pstride = (long long)M * ldc;
  g.err = err;
  if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess ||
      launch_gemm(g, splits, s) != cudaSuccess)
    return kqed::set_error("kqed_bf16_gemm: launch failed");
  int h = 0;
  if (cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return kqed::set_error("kqed_bf16_gemm: execution failed");
  if (h) return kqed::set_error("kqed_bf16_gemm: a tensor-core wait timed out");
  return 0;
}
