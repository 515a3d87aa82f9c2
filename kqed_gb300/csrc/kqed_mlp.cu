/*
 * The learned weight-function surrogate: a 3 -> 256 -> 256 -> 256 -> 39 MLP
 * (SiLU) that maps a generic pair's post-swap invariants (|x|, |y|, cb) to
 * the 39 weight functions the record kernels otherwise interpolate from the
 * form-factor grid (extractff2 / getff7, src/LIBFILES/getff-new.c:262-312,
 * src/LIBFILES/simd.c:488-612; interp_generic here).
 *
 * Training and evaluation run on the GPU through this project's kernels:
 * the first layer (K = 3) in FP32 on the CUDA cores, the three 256-wide
 * products on the tensor cores (kqed_mlp_gemm.cu: BF16 operands, FP32
 * accumulation in tensor memory), backward products and weight gradients
 * through the same GEMM, weight gradients reduced over K splits in a fixed
 * order, Adam on FP32 master weights with BF16 copies for the products.
 *
 * Targets.  The weight functions span 1e-4 .. 1e5 across the grid (their x
 * and y derivatives grow towards small |x|, |y|), so the network predicts
 *   t_i = W_i / (os_i |x|^oa_i |y|^ob_i)
 * with the power law fitted to the training labels (least squares of
 * ln |W_i| on ln |x|, ln |y|) and os_i the RMS of the rescaled values: a
 * cheap base that takes the dynamic range out, leaving O(1) targets.
 *
 * Error bounds.  After training, every held-out sample's error
 * max_i |t_i(net) - t_i(interp)| (the weight-function error in units of its
 * local scale) is binned by cell of feature space; the largest error seen
 * in a cell is its bound.  At evaluation a pair uses the network only when
 * its cell's bound is <= tau; every other pair falls back to the
 * interpolation, which is also the judge of the network's error.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/kqed.h"
#include "kqed_internal.h"
#include "kqed_mlp.h"

namespace kqed {
namespace mlp {

constexpr int H = kH, NIN = kNin, NO = kNo, NOP = kNop;
static_assert(kNo == kSurOut && kNop == kSurOutPad, "surrogate widths");
constexpr size_t oW1 = kOW1, ob1 = kOB1, oW2 = kOW2, ob2 = kOB2, oW3 = kOW3, ob3 = kOB3,
                 oW4 = kOW4, ob4 = kOB4, kParams = kParamCount;
constexpr int kSplits = 32;    /* K splits of the weight-gradient products */

/* ------------------------------------------------------------- kernels */

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + __expf(-z)); }

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(uint64_t seed, uint64_t i, int j)
{
  return (double)(mix64(seed ^ mix64(i * 4 + j)) >> 11) * (1.0 / 9007199254740992.0);
}

/* training samples: |x|, |y| log-uniform on the grid's ranges, cb uniform
   on [-1, 1] */
__global__ void sample_kernel(uint64_t seed, size_t n, double lx0, double lx1, double ly0,
                              double ly1, double *u)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    u[3 * i + 0] = exp(lx0 + (lx1 - lx0) * u01(seed, i, 0));
    u[3 * i + 1] = exp(ly0 + (ly1 - ly0) * u01(seed, i, 1));
    u[3 * i + 2] = 2.0 * u01(seed, i, 2) - 1.0;
  }
}

struct Norm {
  float lo[3], sc[3];
  float oa[NO], ob[NO], os[NO];
};

/* features and normalised targets from invariants and labels */
__global__ void prep_kernel(const double *u, const double *W, size_t n, Norm nm, float4 *feat,
                            float *T)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double lx = log(u[3 * i]), ly = log(u[3 * i + 1]), cb = u[3 * i + 2];
    feat[i] = make_float4(((float)lx - nm.lo[0]) * nm.sc[0] - 1.0f,
                          ((float)ly - nm.lo[1]) * nm.sc[1] - 1.0f,
                          ((float)cb - nm.lo[2]) * nm.sc[2] - 1.0f, 0.0f);
    for (int j = 0; j < NO; j++)
      T[i * 40 + j] = (float)(W[i * NO + j] * exp(-(double)nm.oa[j] * lx - (double)nm.ob[j] * ly) /
                              (double)nm.os[j]);
    T[i * 40 + 39] = 0.0f;
  }
}

/* weight functions from network outputs: W_i = y_i os_i x^oa_i y^ob_i */
__global__ void denorm_kernel(const float *Y, const double *u, size_t n, Norm nm, float *W)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float lx = (float)log(u[3 * i]), ly = (float)log(u[3 * i + 1]);
    for (int j = 0; j < NO; j++)
      W[i * NO + j] = Y[i * NOP + j] * nm.os[j] * __expf(nm.oa[j] * lx + nm.ob[j] * ly);
  }
}

/* layer 1 (3 -> 256) on the CUDA cores: Z1 = W1 f + b1, H1 = bf16(silu(Z1)) */
__global__ void layer1_kernel(const float4 *feat, const unsigned *countp, size_t rows,
                              const float *P, float *Z1, __nv_bfloat16 *H1)
{
  const size_t n = countp ? min(rows, (size_t)*countp) : rows;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * H;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t b = e / H;
    const int j = (int)(e % H);
    const float4 f = feat[b];
    const float *w = P + oW1 + 3 * j;
    const float z = fmaf(w[2], f.z, fmaf(w[1], f.y, fmaf(w[0], f.x, P[ob1 + j])));
    if (Z1) Z1[e] = z;
    H1[e] = __float2bfloat16_rn(silu_f(z));
  }
}

/* mean-square loss over the 39 outputs and its gradient */
__global__ void loss_grad_kernel(const float *Y, const float *T, int B, float *dYf,
                                 __nv_bfloat16 *dYb, float *lossp)
{
  __shared__ float red[256];
  float acc = 0.0f;
  const float sc = 2.0f / ((float)B * (float)NO);
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    for (int j = 0; j < NOP; j++) {
      float d = 0.0f;
      if (j < NO) {
        d = Y[(size_t)b * NOP + j] - T[(size_t)b * 40 + j];
        acc += d * d;
      }
      dYf[(size_t)b * NOP + j] = sc * d;
      dYb[(size_t)b * NOP + j] = __float2bfloat16_rn(sc * d);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) lossp[blockIdx.x] = red[0];
}

/* out[j] = sum_b D[b][j] (block per column, fixed order) */
__global__ void colsum_kernel(const float *D, int B, int ld, float *out)
{
  __shared__ float red[256];
  const int j = blockIdx.x;
  float s = 0.0f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) s += D[(size_t)b * ld + j];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = red[0];
}

/* gradient of layer 1: gW1[j][i] = sum_b dZ1[b][j] f_i, gb1[j] = sum_b dZ1[b][j] */
__global__ void layer1_grad_kernel(const float *dZ1, const float4 *feat, int B, float *G)
{
  __shared__ float red[4][256];
  const int j = blockIdx.x;
  float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const float d = dZ1[(size_t)b * H + j];
    const float4 f = feat[b];
    s[0] += d * f.x; s[1] += d * f.y; s[2] += d * f.z; s[3] += d;
  }
  for (int q = 0; q < 4; q++) red[q][threadIdx.x] = s[q];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int q = 0; q < 4; q++) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < 3; i++) G[oW1 + 3 * j + i] = red[i][0];
    G[ob1 + j] = red[3][0];
  }
}

/* out[e] = sum_s part[s * pstride + e], in split order */
__global__ void reduce_splits_kernel(const float *part, int S, size_t n, size_t pstride, float *out)
{
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int z = 0; z < S; z++) s += part[(size_t)z * pstride + e];
    out[e] = s;
  }
}

/* Adam (Kingma & Ba) on the FP32 master weights */
__global__ void adam_kernel(float *P, const float *G, float *M, float *V, size_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float g = G[i];
    const float m = b1 * M[i] + (1.0f - b1) * g;
    const float v = b2 * V[i] + (1.0f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
  }
}

/* BF16 copies of the three tensor-core weight matrices */
__global__ void weights_bf16_kernel(const float *P, __nv_bfloat16 *W2h, __nv_bfloat16 *W3h,
                                    __nv_bfloat16 *W4h)
{
  const size_t n2 = (size_t)H * H, n4 = (size_t)NOP * H;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < 2 * n2 + n4;
       e += (size_t)gridDim.x * blockDim.x) {
    if (e < n2) W2h[e] = __float2bfloat16_rn(P[oW2 + e]);
    else if (e < 2 * n2) W3h[e - n2] = __float2bfloat16_rn(P[oW3 + e - n2]);
    else {
      const size_t q = e - 2 * n2;
      W4h[q] = __float2bfloat16_rn((q / H) < (size_t)NO ? P[oW4 + q] : 0.0f);
    }
  }
}

/* per-sample error in target units, binned by feature cell (atomic max of
   non-negative floats through their bit patterns): cell[c] over the 37
   weight functions every generic pair uses, cell[ncell + c] also over the
   two y-derivative differences only swapped pairs use; totals of the 37
   for the RMS */
__global__ void cell_error_kernel(const float *Y, const float *T, const float4 *feat, size_t n,
                                  int nb0, int nb1, int nb2, unsigned *cell, double *sums)
{
  double sq = 0.0;
  float mx = 0.0f;
  const size_t ncell = (size_t)nb0 * nb1 * nb2;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float e = 0.0f, e2 = 0.0f;
    for (int j = 0; j < NO; j++) {
      const float d = fabsf(Y[i * NOP + j] - T[i * 40 + j]);
      if (j < 37) {
        e = fmaxf(e, d);
        sq += (double)d * d;
      } else {
        e2 = fmaxf(e2, d);
      }
    }
    const float4 f = feat[i];
    const int c0 = min(nb0 - 1, max(0, (int)((f.x + 1.0f) * 0.5f * nb0)));
    const int c1 = min(nb1 - 1, max(0, (int)((f.y + 1.0f) * 0.5f * nb1)));
    const int c2 = min(nb2 - 1, max(0, (int)((f.z + 1.0f) * 0.5f * nb2)));
    const size_t c = ((size_t)c0 * nb1 + c1) * nb2 + c2;
    atomicMax(cell + c, __float_as_uint(e));
    atomicMax(cell + ncell + c, __float_as_uint(fmaxf(e, e2)));
    mx = fmaxf(mx, e);
  }
  atomicAdd(sums, sq);
  atomicMax(reinterpret_cast<unsigned *>(sums + 1), __float_as_uint(mx));
}

static unsigned grid_for(size_t n, int threads = 256)
{
  return (unsigned)std::max<size_t>(1, std::min<size_t>((n + threads - 1) / threads, 152 * 16));
}

/* ------------------------------------------------------------- network */

struct Net {
  float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;
  __nv_bfloat16 *W2h = nullptr, *W3h = nullptr, *W4h = nullptr;
  __nv_bfloat16 *wimg = nullptr;     /* weight image of the fused evaluation kernel */
  int step = 0;
  int alloc()
  {
    if (cudaMalloc(&P, 4 * kParams * sizeof(float)) != cudaSuccess) return 1;
    G = P + kParams;
    M = G + kParams;
    V = M + kParams;
    if (cudaMalloc(&W2h, (2 * (size_t)H * H + (size_t)NOP * H) * sizeof(__nv_bfloat16)) !=
        cudaSuccess)
      return 1;
    W3h = W2h + (size_t)H * H;
    W4h = W3h + (size_t)H * H;
    if (cudaMalloc(&wimg, kWimgBytes) != cudaSuccess) return 1;
    return 0;
  }
  void release()
  {
    if (P) cudaFree(P);
    if (W2h) cudaFree(W2h);
    if (wimg) cudaFree(wimg);
    P = G = M = V = nullptr;
    W2h = W3h = W4h = wimg = nullptr;
  }
};

/* activations of one batch of rows */
struct Work {
  size_t rows = 0;
  float *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr, *Y = nullptr, *dYf = nullptr, *dZf = nullptr;
  float *part = nullptr, *lossp = nullptr;
  __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *dYb = nullptr, *dZa = nullptr,
                *dZb = nullptr;
  void *mem = nullptr;
  int alloc(size_t n, bool train)
  {
    rows = n;
    const size_t f = train ? (3 * n * H + 2 * n * NOP + n * H + (size_t)kSplits * H * H + 1024)
                           : (n * NOP);
    const size_t h = train ? (5 * n * H + n * NOP) : 0;
    if (cudaMalloc(&mem, f * sizeof(float) + h * sizeof(__nv_bfloat16) + 256) != cudaSuccess)
      return 1;
    float *fp = static_cast<float *>(mem);
    if (train) {
      Z1 = fp; fp += n * H;
      Z2 = fp; fp += n * H;
      Z3 = fp; fp += n * H;
      dYf = fp; fp += n * NOP;
      dZf = fp; fp += n * H;
      part = fp; fp += (size_t)kSplits * H * H;
      lossp = fp; fp += 1024;
    }
    Y = fp; fp += n * NOP;
    if (train) {
      __nv_bfloat16 *hp = reinterpret_cast<__nv_bfloat16 *>(fp);
      H1 = hp; hp += n * H;
      H2 = hp; hp += n * H;
      H3 = hp; hp += n * H;
      dZa = hp; hp += n * H;
      dZb = hp; hp += n * H;
      dYb = hp; hp += n * NOP;
    }
    return 0;
  }
  void release()
  {
    if (mem) cudaFree(mem);
    mem = nullptr;
  }
};

static GemmArgs gemm(const __nv_bfloat16 *A, long long sAm, long long sAk, const __nv_bfloat16 *B,
                     long long sBn, long long sBk, int M, int N, int K, int mode, int *err)
{
  GemmArgs g{};
  g.A = A; g.sAm = sAm; g.sAk = sAk;
  g.B = B; g.sBn = sBn; g.sBk = sBk;
  g.M = M; g.N = N; g.K = K;
  g.mode = mode;
  g.err = err;
  return g;
}

#define TRY(x)                                        \
  do {                                                \
    const cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return e_;                 \
  } while (0)

/* Y = net(feat) for the first min(rows, *countp) rows (countp NULL: rows) */
static cudaError_t forward(const Net &N, const float4 *feat, const unsigned *countp, size_t rows,
                           Work &w, bool keepZ, int *err, cudaStream_t s)
{
  layer1_kernel<<<grid_for(rows * H), 256, 0, s>>>(feat, countp, rows, N.P, keepZ ? w.Z1 : nullptr,
                                                   w.H1);
  g_launches++;
  GemmArgs g = gemm(w.H1, H, 1, N.W2h, H, 1, (int)rows, H, H, kHidden, err);
  g.bias = N.P + ob2; g.cf = keepZ ? w.Z2 : nullptr; g.ldc = H; g.cb = w.H2; g.ldb = H;
  g.Mdev = countp;
  TRY(launch_gemm(g, 1, s));
  g = gemm(w.H2, H, 1, N.W3h, H, 1, (int)rows, H, H, kHidden, err);
  g.bias = N.P + ob3; g.cf = keepZ ? w.Z3 : nullptr; g.ldc = H; g.cb = w.H3; g.ldb = H;
  g.Mdev = countp;
  TRY(launch_gemm(g, 1, s));
  g = gemm(w.H3, H, 1, N.W4h, H, 1, (int)rows, NOP, H, kOut, err);
  g.bias = N.P + ob4; g.cf = w.Y; g.ldc = NOP;
  g.Mdev = countp;
  TRY(launch_gemm(g, 1, s));
  return cudaGetLastError();
}

/* Y = net(feat) by the fused evaluation kernel (the weight image must be
   current: launch_build_wimg after the parameters change) */
static cudaError_t infer(const Net &N, const float4 *feat, const unsigned *countp, size_t rows,
                         float *Y, int *err, cudaStream_t s)
{
  InferArgs a{feat, countp, rows, N.P, N.wimg, Y, err};
  return launch_mlp_infer(a, s);
}

/* gradient of the mean-square loss at the current weights into N.G */
static cudaError_t backward(const Net &N, const float4 *feat, const float *T, int B, Work &w,
                            int *err, cudaStream_t s)
{
  const int lb = (int)std::min<size_t>((B + 255) / 256, 1024);
  loss_grad_kernel<<<lb, 256, 0, s>>>(w.Y, T, B, w.dYf, w.dYb, w.lossp);
  /* output layer */
  GemmArgs g = gemm(w.dYb, 1, NOP, w.H3, 1, H, NOP, H, B, kStore, err);
  g.cf = w.part; g.ldc = H; g.pstride = (long long)H * H;
  TRY(launch_gemm(g, kSplits, s));
  reduce_splits_kernel<<<grid_for((size_t)NOP * H), 256, 0, s>>>(w.part, kSplits, (size_t)NOP * H,
                                                                   (size_t)H * H, N.G + oW4);
  colsum_kernel<<<NOP, 256, 0, s>>>(w.dYf, B, NOP, N.G + ob4);
  /* dZ3 = (dY W4) * silu'(Z3) */
  g = gemm(w.dYb, NOP, 1, N.W4h, 1, H, B, H, NOP, kBwd, err);
  g.zin = w.Z3; g.cf = w.dZf; g.ldc = H; g.cb = w.dZa; g.ldb = H;
  TRY(launch_gemm(g, 1, s));
  colsum_kernel<<<H, 256, 0, s>>>(w.dZf, B, H, N.G + ob3);
  g = gemm(w.dZa, 1, H, w.H2, 1, H, H, H, B, kStore, err);
  g.cf = w.part; g.ldc = H; g.pstride = (long long)H * H;
  TRY(launch_gemm(g, kSplits, s));
  reduce_splits_kernel<<<grid_for((size_t)H * H), 256, 0, s>>>(w.part, kSplits, (size_t)H * H,
                                                                 (size_t)H * H, N.G + oW3);
  /* dZ2 = (dZ3 W3) * silu'(Z2) */
  g = gemm(w.dZa, H, 1, N.W3h, 1, H, B, H, H, kBwd, err);
  g.zin = w.Z2; g.cf = w.dZf; g.ldc = H; g.cb = w.dZb; g.ldb = H;
  TRY(launch_gemm(g, 1, s));
  colsum_kernel<<<H, 256, 0, s>>>(w.dZf, B, H, N.G + ob2);
  g = gemm(w.dZb, 1, H, w.H1, 1, H, H, H, B, kStore, err);
  g.cf = w.part; g.ldc = H; g.pstride = (long long)H * H;
  TRY(launch_gemm(g, kSplits, s));
  reduce_splits_kernel<<<grid_for((size_t)H * H), 256, 0, s>>>(w.part, kSplits, (size_t)H * H,
                                                                 (size_t)H * H, N.G + oW2);
  /* dZ1 = (dZ2 W2) * silu'(Z1), then layer 1 on the CUDA cores */
  g = gemm(w.dZb, H, 1, N.W2h, 1, H, B, H, H, kBwd, err);
  g.zin = w.Z1; g.cf = w.dZf; g.ldc = H; g.cb = nullptr;
  TRY(launch_gemm(g, 1, s));
  layer1_grad_kernel<<<H, 256, 0, s>>>(w.dZf, feat, B, N.G);
  g_launches += 8;
  return cudaGetLastError();
}

static cudaError_t adam_step(Net &N, float lr, cudaStream_t s)
{
  N.step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f / (1.0f - powf(b1, (float)N.step));
  const float c2 = 1.0f / (1.0f - powf(b2, (float)N.step));
  adam_kernel<<<grid_for(kParams), 256, 0, s>>>(N.P, N.G, N.M, N.V, kParams, lr, b1, b2, 1e-8f,
                                                c1, c2);
  weights_bf16_kernel<<<grid_for(2 * (size_t)H * H), 256, 0, s>>>(N.P, N.W2h, N.W3h, N.W4h);
  g_launches += 2;
  return cudaGetLastError();
}

static cudaError_t upload_params(Net &N, const float *host, cudaStream_t s)
{
  TRY(cudaMemcpyAsync(N.P, host, kParams * sizeof(float), cudaMemcpyHostToDevice, s));
  TRY(cudaMemsetAsync(N.M, 0, 2 * kParams * sizeof(float), s));
  weights_bf16_kernel<<<grid_for(2 * (size_t)H * H), 256, 0, s>>>(N.P, N.W2h, N.W3h, N.W4h);
  g_launches++;
  N.step = 0;
  return cudaGetLastError();
}

/* He-uniform initial weights (seeded), zero biases */
static void init_params(std::vector<float> &p, uint64_t seed)
{
  p.assign(kParams, 0.0f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 12345;
  auto uni = [&st]() {
    st ^= st >> 12; st ^= st << 25; st ^= st >> 27;
    return (double)((st * 2685821657736338717ull) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  };
  auto fill = [&](size_t off, size_t n, double a) {
    for (size_t i = 0; i < n; i++) p[off + i] = (float)(a * uni());
  };
  fill(oW1, (size_t)H * NIN, std::sqrt(6.0 / NIN));
  fill(oW2, (size_t)H * H, std::sqrt(6.0 / H));
  fill(oW3, (size_t)H * H, std::sqrt(6.0 / H));
  fill(oW4, (size_t)NO * H, std::sqrt(1.0 / H));
}

/* ------------------------------------------------------ trained surrogate */

struct Surrogate {
  int device = 0;
  Net net;
  Norm norm{};
  int nb[3] = {24, 24, 16};
  std::vector<float> cell_host;      /* [2][ncell] */
  float *cell_dev = nullptr;
  float tau = 1e-3f;
  SurDev *sdev = nullptr;            /* device struct of the lattice launches */
  /* evaluation scratch of the lattice launches (grown on demand) */
  Work ework;
  float4 *efeat = nullptr;
  uint32_t *elist = nullptr;
  unsigned *ecount = nullptr;
  size_t ecap = 0;
  int *err = nullptr;
  ~Surrogate()
  {
    net.release();
    ework.release();
    if (cell_dev) cudaFree(cell_dev);
    if (sdev) cudaFree(sdev);
    if (efeat) cudaFree(efeat);
    if (elist) cudaFree(elist);
    if (ecount) cudaFree(ecount);
  }
};

/* RMS and max of the held-out error (target units, the 37 weight functions
   of every pair); with cell != NULL the per-cell maxima as well */
static cudaError_t evaluate(const Net &N, const float4 *feat, const float *T, size_t n,
                            const int nb[3], unsigned *cell, double *rms, double *mx, int *err,
                            cudaStream_t s)
{
  const size_t chunk = 65536;
  Work w;
  if (w.alloc(chunk, false)) return cudaErrorMemoryAllocation;
  TRY(launch_build_wimg(N.P, N.wimg, s));
  double *sums = nullptr;
  cudaError_t e = cudaMalloc(&sums, 2 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(sums, 0, 2 * sizeof(double), s);
  unsigned *scratch_cell = nullptr;
  if (e == cudaSuccess && !cell) {
    e = cudaMalloc(&scratch_cell, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch_cell, 0, 2 * sizeof(unsigned), s);
  }
  for (size_t o = 0; e == cudaSuccess && o < n; o += chunk) {
    const size_t m = std::min(chunk, n - o);
    e = infer(N, feat + o, nullptr, m, w.Y, err, s);
    if (e != cudaSuccess) break;
    if (cell)
      cell_error_kernel<<<grid_for(m), 256, 0, s>>>(w.Y, T + 40 * o, feat + o, m, nb[0], nb[1],
                                                    nb[2], cell, sums);
    else
      cell_error_kernel<<<grid_for(m), 256, 0, s>>>(w.Y, T + 40 * o, feat + o, m, 1, 1, 1,
                                                    scratch_cell, sums);
    g_launches++;
    e = cudaGetLastError();
  }
  double h[2] = {0.0, 0.0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  unsigned bits;
  std::memcpy(&bits, &h[1], sizeof(unsigned));
  float fm;
  std::memcpy(&fm, &bits, sizeof(float));
  *rms = std::sqrt(h[0] / std::max<double>(1.0, (double)n * 37));
  *mx = fm;
  w.release();
  if (sums) cudaFree(sums);
  if (scratch_cell) cudaFree(scratch_cell);
  return e;
}

std::mutex g_mu;
std::map<const void *, Surrogate *> g_sur;

Surrogate *find(const void *ctx)
{
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_sur.find(ctx);
  return it == g_sur.end() ? nullptr : it->second;
}

void attach(const void *ctx, Surrogate *s)
{
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_sur.find(ctx);
  if (it != g_sur.end()) delete it->second;
  g_sur[ctx] = s;
}

/* power law and scale of the targets from a sample of labels (host) */
static void fit_norm(const std::vector<double> &u, const std::vector<double> &W, size_t n, Norm &nm)
{
  for (int j = 0; j < NO; j++) {
    /* least squares of ln|W_j| = a ln x + b ln y + c */
    double A[3][3] = {}, rhs[3] = {};
    for (size_t i = 0; i < n; i++) {
      const double w = std::fabs(W[i * NO + j]);
      if (!(w > 0.0) || !std::isfinite(w)) continue;
      const double v[3] = {std::log(u[3 * i]), std::log(u[3 * i + 1]), 1.0};
      const double lw = std::log(w);
      for (int a = 0; a < 3; a++) {
        rhs[a] += v[a] * lw;
        for (int b = 0; b < 3; b++) A[a][b] += v[a] * v[b];
      }
    }
    /* 3x3 solve by Cramer's rule */
    auto det3 = [](double M[3][3]) {
      return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
             M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
             M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    };
    const double d = det3(A);
    double sol[3] = {0.0, 0.0, 0.0};
    if (std::fabs(d) > 0.0)
      for (int c = 0; c < 3; c++) {
        double M[3][3];
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) M[a][b] = (b == c) ? rhs[a] : A[a][b];
        sol[c] = det3(M) / d;
      }
    nm.oa[j] = (float)sol[0];
    nm.ob[j] = (float)sol[1];
    double ss = 0.0;
    size_t cnt = 0;
    for (size_t i = 0; i < n; i++) {
      const double r = W[i * NO + j] * std::exp(-(double)nm.oa[j] * std::log(u[3 * i]) -
                                                (double)nm.ob[j] * std::log(u[3 * i + 1]));
      if (std::isfinite(r)) { ss += r * r; cnt++; }
    }
    const double rms = cnt ? std::sqrt(ss / cnt) : 1.0;
    nm.os[j] = (float)(rms > 0.0 ? rms : 1.0);
  }
}

static cudaError_t surrogate_device_struct(Surrogate &S)
{
  SurDev d{};
  d.cell = S.cell_dev;
  for (int i = 0; i < 3; i++) {
    d.nb[i] = S.nb[i];
    d.lo[i] = S.norm.lo[i];
    d.sc[i] = S.norm.sc[i];
  }
  d.tau = S.tau;
  for (int j = 0; j < NO; j++) {
    d.oa[j] = S.norm.oa[j];
    d.ob[j] = S.norm.ob[j];
    d.os[j] = S.norm.os[j];
  }
  d.feat = S.efeat;
  d.elist = S.elist;
  d.ecount = S.ecount;
  d.etotal = reinterpret_cast<unsigned long long *>(S.ecount + 2);
  d.Y = S.ework.Y;
  if (!S.sdev) TRY(cudaMalloc(&S.sdev, sizeof(SurDev)));
  return cudaMemcpy(S.sdev, &d, sizeof(SurDev), cudaMemcpyHostToDevice);
}

static int train(const DevTables &T, const kqed_surrogate_opts &o, kqed_surrogate_report *rep,
                 Surrogate **out)
{
  const auto t0 = std::chrono::steady_clock::now();
  const size_t n = o.samples, nh = o.heldout, ntot = n + nh;
  const int B = o.batch;
  if (n < (size_t)B || B < 256 || B % 128 || nh == 0 || o.epochs < 1)
    return set_error("kqed_surrogate_train: need samples >= batch, batch a multiple of 128 "
                     ">= 256, heldout > 0, epochs >= 1");
  Surrogate *S = new Surrogate();
  cudaGetDevice(&S->device);
  cudaStream_t s = nullptr;
  double *u = nullptr, *Wc = nullptr;
  float4 *feat = nullptr;
  float *Tg = nullptr;
  unsigned *cell = nullptr;
  Work w;
  int rc = 0;
  auto bail = [&](const char *msg) {
    rc = set_error(msg);
    return rc;
  };
  do {
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { bail("stream"); break; }
    if (device_error_flag(&S->err) || cudaMemsetAsync(S->err, 0, sizeof(int), s) != cudaSuccess) {
      bail("kqed_surrogate_train: error flag");
      break;
    }
    double g[4];
    const int nx = T.nstpx, ny = T.nstpy;
    if (cudaMemcpy(&g[0], T.XX, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&g[1], T.XX + nx - 1, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&g[2], T.YY, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&g[3], T.YY + ny - 1, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
      bail("kqed_surrogate_train: grid");
      break;
    }
    const double lx0 = std::log(g[0]), lx1 = std::log(g[1]), ly0 = std::log(g[2]),
                 ly1 = std::log(g[3]);
    Norm &nm = S->norm;
    nm.lo[0] = (float)lx0; nm.sc[0] = (float)(2.0 / (lx1 - lx0));
    nm.lo[1] = (float)ly0; nm.sc[1] = (float)(2.0 / (ly1 - ly0));
    nm.lo[2] = -1.0f; nm.sc[2] = 1.0f;
    const size_t chunk = (size_t)1 << 20;
    if (cudaMalloc(&u, ntot * 3 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&Wc, chunk * NO * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&feat, ntot * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&Tg, ntot * 40 * sizeof(float)) != cudaSuccess) {
      bail("kqed_surrogate_train: out of device memory for the samples");
      break;
    }
    sample_kernel<<<grid_for(ntot), 256, 0, s>>>(o.seed, ntot, lx0, lx1, ly0, ly1, u);
    g_launches++;
    /* the target scaling from the first labels */
    {
      const size_t m = std::min<size_t>(ntot, 262144);
      if (launch_weight_labels(T, u, m, Wc, s) != cudaSuccess) { bail("labels"); break; }
      std::vector<double> hu(3 * m), hw((size_t)NO * m);
      if (cudaMemcpyAsync(hu.data(), u, hu.size() * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaMemcpyAsync(hw.data(), Wc, hw.size() * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) {
        bail("kqed_surrogate_train: label sample");
        break;
      }
      fit_norm(hu, hw, m, nm);
    }
    bool ok = true;
    for (size_t o0 = 0; o0 < ntot && ok; o0 += chunk) {
      const size_t m = std::min(chunk, ntot - o0);
      ok = launch_weight_labels(T, u + 3 * o0, m, Wc, s) == cudaSuccess;
      prep_kernel<<<grid_for(m), 256, 0, s>>>(u + 3 * o0, Wc, m, nm, feat + o0, Tg + 40 * o0);
      g_launches++;
    }
    if (!ok || cudaGetLastError() != cudaSuccess) { bail("kqed_surrogate_train: labels"); break; }
    /* network */
    if (S->net.alloc() || w.alloc((size_t)B, true)) { bail("kqed_surrogate_train: out of memory"); break; }
    std::vector<float> p0;
    init_params(p0, o.seed + 1);
    if (upload_params(S->net, p0.data(), s) != cudaSuccess) { bail("upload"); break; }
    double urms = 0.0, umax = 0.0;
    if (evaluate(S->net, feat + n, Tg + 40 * n, nh, S->nb, nullptr, &urms, &umax, S->err, s) !=
        cudaSuccess) {
      bail("kqed_surrogate_train: evaluation failed");
      break;
    }
    const size_t spe = n / (size_t)B;
    const size_t total = spe * (size_t)o.epochs;
    const auto tt0 = std::chrono::steady_clock::now();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    double loss_sum = 0.0;
    int loss_n = 0;
    std::vector<float> lp(1024);
    const int lb = (int)std::min<size_t>(((size_t)B + 255) / 256, 1024);
    for (size_t st = 0; st < total && ok; st++) {
      const size_t off = (st % spe) * (size_t)B;
      const double warm = 200.0;
      const double fr = (double)st / (double)std::max<size_t>(total - 1, 1);
      double lr = o.lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(3.141592653589793 * fr)));
      if ((double)st < warm) lr *= ((double)st + 1.0) / warm;
      ok = forward(S->net, feat + off, nullptr, (size_t)B, w, true, S->err, s) == cudaSuccess &&
           backward(S->net, feat + off, Tg + 40 * off, B, w, S->err, s) == cudaSuccess &&
           adam_step(S->net, (float)lr, s) == cudaSuccess;
      if (ok && st + 20 >= total) {
        ok = cudaMemcpyAsync(lp.data(), w.lossp, lb * sizeof(float), cudaMemcpyDeviceToHost, s) ==
                 cudaSuccess &&
             cudaStreamSynchronize(s) == cudaSuccess;
        double l = 0.0;
        for (int i = 0; i < lb; i++) l += lp[i];
        loss_sum += l / ((double)B * NO);
        loss_n++;
      }
    }
    cudaEventRecord(e1, s);
    if (!ok || cudaStreamSynchronize(s) != cudaSuccess) { bail("kqed_surrogate_train: training step failed"); break; }
    float train_ms = 0.0f;
    cudaEventElapsedTime(&train_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double train_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - tt0).count();
    /* per-cell bounds on the held-out samples */
    const size_t ncell = (size_t)S->nb[0] * S->nb[1] * S->nb[2];
    if (cudaMalloc(&cell, 2 * ncell * sizeof(unsigned)) != cudaSuccess ||
        cudaMemsetAsync(cell, 0, 2 * ncell * sizeof(unsigned), s) != cudaSuccess) {
      bail("kqed_surrogate_train: cells");
      break;
    }
    double hrms = 0.0, hmax = 0.0;
    if (evaluate(S->net, feat + n, Tg + 40 * n, nh, S->nb, cell, &hrms, &hmax, S->err, s) !=
        cudaSuccess) {
      bail("kqed_surrogate_train: evaluation failed");
      break;
    }
    std::vector<unsigned> cb(2 * ncell);
    if (cudaMemcpy(cb.data(), cell, 2 * ncell * sizeof(unsigned), cudaMemcpyDeviceToHost) !=
        cudaSuccess) {
      bail("cells");
      break;
    }
    S->cell_host.resize(2 * ncell);
    size_t acc = 0;
    S->tau = (float)o.tau;
    for (size_t i = 0; i < 2 * ncell; i++) {
      float f;
      std::memcpy(&f, &cb[i], sizeof(float));
      /* a cell no held-out sample reached gets no bound */
      S->cell_host[i] = cb[i] ? f : 3.0e38f;
      if (i < ncell) acc += S->cell_host[i] <= S->tau;
    }
    if (cudaMalloc(&S->cell_dev, 2 * ncell * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(S->cell_dev, S->cell_host.data(), 2 * ncell * sizeof(float),
                   cudaMemcpyHostToDevice) != cudaSuccess) {
      bail("cells");
      break;
    }
    int herr = 0;
    cudaMemcpy(&herr, S->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (herr) { bail("kqed_surrogate_train: a tensor-core wait timed out"); break; }
    if (rep) {
      rep->loss_final = loss_n ? loss_sum / loss_n : 0.0;
      rep->heldout_rms = hrms;
      rep->heldout_max = hmax;
      rep->untrained_rms = urms;
      rep->untrained_max = umax;
      rep->train_seconds = train_s;
      rep->steps = (double)total;
      rep->cells_accepted = ncell ? (double)acc / (double)ncell : 0.0;
      /* tensor-core work per step: 3 forward products, 3 data-gradient and
         3 weight-gradient products (2 flops per multiply-add) */
      const double per_row = 2.0 * ((double)H * H * 2 + (double)H * NOP);
      rep->gemm_tflops = 3.0 * per_row * (double)B * (double)total / (train_ms * 1e-3) / 1e12;
      rep->seconds_total =
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
  } while (0);
  w.release();
  if (u) cudaFree(u);
  if (Wc) cudaFree(Wc);
  if (feat) cudaFree(feat);
  if (Tg) cudaFree(Tg);
  if (cell) cudaFree(cell);
  if (s) cudaStreamDestroy(s);
  if (rc) {
    delete S;
    return rc;
  }
  *out = S;
  return 0;
}

/* the lattice hook: the network over the first *ecount of `rows` selected pairs */
static cudaError_t run_hook(void *state, size_t rows, cudaStream_t s)
{
  Surrogate *S = static_cast<Surrogate *>(state);
  return infer(S->net, S->efeat, S->ecount, rows, S->ework.Y, S->err, s);
}

/* evaluation buffers for `cap` selected pairs */
static int ensure_capacity(Surrogate &S, size_t cap)
{
  if (cap <= S.ecap && S.sdev) return 0;
  S.ework.release();
  if (S.efeat) cudaFree(S.efeat);
  if (S.elist) cudaFree(S.elist);
  S.efeat = nullptr;
  S.elist = nullptr;
  /* the per-chunk count, then (8-byte aligned) the running total */
  if (!S.ecount) {
    if (cudaMalloc(&S.ecount, 4 * sizeof(unsigned)) != cudaSuccess) return 1;
    if (cudaMemset(S.ecount, 0, 4 * sizeof(unsigned)) != cudaSuccess) return 1;
  }
  if (cudaMalloc(&S.efeat, cap * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&S.elist, cap * sizeof(uint32_t)) != cudaSuccess || S.ework.alloc(cap, false))
    return 1;
  S.ecap = cap;
  return surrogate_device_struct(S) != cudaSuccess;
}

} // namespace mlp

/* called by free_QED_temps: a later context may reuse the address */
void surrogate_forget(const void *ctx)
{
  std::lock_guard<std::mutex> g(mlp::g_mu);
  auto it = mlp::g_sur.find(ctx);
  if (it != mlp::g_sur.end()) {
    delete it->second;
    mlp::g_sur.erase(it);
  }
}

bool surrogate_ready(const void *ctx) { return mlp::find(ctx) != nullptr; }

int surrogate_hook(const void *ctx, size_t cap, SurHook *hook)
{
  mlp::Surrogate *S = mlp::find(ctx);
  if (!S) return set_error("no surrogate: train or load one for these tables first");
  if (mlp::ensure_capacity(*S, cap)) return set_error("out of device memory for the surrogate");
  hook->d = S->sdev;
  hook->ecount = S->ecount;
  hook->run = mlp::run_hook;
  hook->state = S;
  return 0;
}

} // namespace kqed

using namespace kqed;

extern "C" int kqed_surrogate_train(const struct QED_kernel_temps *t,
                                    const struct kqed_surrogate_opts *opts,
                                    struct kqed_surrogate_report *report)
{
  DevTables T;
  DevMaps M;
  LaunchCfg cfg;
  if (ctx_handles(t, &T, &M, &cfg)) return set_error("tables not initialised");
  kqed_surrogate_opts o{};
  o.samples = 10000000;
  o.heldout = 1000000;
  o.batch = 8192;
  o.epochs = 4;
  o.lr = 2e-3;
  o.seed = 5;
  o.tau = 1e-3;
  if (opts) o = *opts;
  mlp::Surrogate *S = nullptr;
  if (mlp::train(T, o, report, &S)) return 1;
  if (mlp::surrogate_device_struct(*S) != cudaSuccess) {
    delete S;
    return set_error("kqed_surrogate_train: device struct");
  }
  mlp::attach(t->Grid.PC->Fm, S);
  return 0;
}

extern "C" int kqed_surrogate_set_tolerance(const struct QED_kernel_temps *t, double tau)
{
  if (!t || !t->Grid.PC) return set_error("tables not initialised");
  mlp::Surrogate *S = mlp::find(t->Grid.PC->Fm);
  if (!S) return set_error("no surrogate: train one for these tables first");
  S->tau = (float)std::min(tau, 3.0e38);
  if (mlp::surrogate_device_struct(*S) != cudaSuccess) return set_error("device struct");
  return 0;
}

extern "C" int kqed_surrogate_cells(const struct QED_kernel_temps *t, double tau,
                                    double *accepted_fraction)
{
  if (!t || !t->Grid.PC) return set_error("tables not initialised");
  mlp::Surrogate *S = mlp::find(t->Grid.PC->Fm);
  if (!S) return set_error("no surrogate: train one for these tables first");
  const size_t nc = S->cell_host.size() / 2;
  size_t a = 0;
  for (size_t i = 0; i < nc; i++) a += S->cell_host[i] <= tau;
  *accepted_fraction = nc ? (double)a / (double)nc : 0.0;
  return 0;
}

/* network and interpolation at given post-swap invariants (device buffers):
   d_wnet[i][39] from the trained network, d_winterp[i][39] (optional) from
   the FP64 interpolation */
extern "C" int kqed_surrogate_weights(const struct QED_kernel_temps *t, size_t n, const double *d_u,
                                      float *d_wnet, double *d_winterp, void *stream)
{
  DevTables T;
  DevMaps M;
  LaunchCfg cfg;
  if (ctx_handles(t, &T, &M, &cfg)) return set_error("tables not initialised");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (d_winterp && launch_weight_labels(T, d_u, n, d_winterp, s) != cudaSuccess)
    return set_error("kqed_surrogate_weights: labels failed");
  if (!d_wnet || n == 0) {
    if (cudaStreamSynchronize(s) != cudaSuccess) return set_error("kqed_surrogate_weights: failed");
    return 0;
  }
  mlp::Surrogate *S = mlp::find(t->Grid.PC->Fm);
  if (!S) return set_error("no surrogate: train one for these tables first");
  double *W = nullptr;
  mlp::Work w;
  float4 *feat = nullptr;
  float *Tg = nullptr;
  int rc = 0;
  if (cudaMalloc(&W, n * mlp::NO * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&feat, n * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&Tg, n * 40 * sizeof(float)) != cudaSuccess || w.alloc(n, false))
    rc = set_error("kqed_surrogate_weights: out of memory");
  if (!rc) {
    if (launch_weight_labels(T, d_u, n, W, s) != cudaSuccess) {
      rc = set_error("kqed_surrogate_weights: labels failed");
    } else {
      mlp::prep_kernel<<<mlp::grid_for(n), 256, 0, s>>>(d_u, W, n, S->norm, feat, Tg);
      g_launches++;
      if (cudaGetLastError() != cudaSuccess ||
          mlp::infer(S->net, feat, nullptr, n, w.Y, S->err, s) != cudaSuccess)
        rc = set_error("kqed_surrogate_weights: evaluation failed");
    }
  }
  if (!rc) {
    mlp::denorm_kernel<<<mlp::grid_for(n), 256, 0, s>>>(w.Y, d_u, n, S->norm, d_wnet);
    g_launches++;
    if (cudaStreamSynchronize(s) != cudaSuccess) rc = set_error("kqed_surrogate_weights: failed");
  }
  w.release();
  if (W) cudaFree(W);
  if (feat) cudaFree(feat);
  if (Tg) cudaFree(Tg);
  return rc;
}

/* One forward and backward pass of the network on host data, no update
   (the gradient check): params[kParams] fp32, feat[n][3], target[n][39]
   (target units); y[n][39] network outputs, grad[kParams], loss. */
extern "C" int kqed_mlp_forward_backward(const float *params, size_t n, const float *feat,
                                         const float *target, float *y, float *grad,
                                         double *loss)
{
  using namespace mlp;
  if (!params || !feat || !target || n == 0 || n % 128)
    return set_error("kqed_mlp_forward_backward: n must be a positive multiple of 128");
  Net N;
  Work w;
  float4 *df = nullptr;
  float *dt = nullptr;
  int *err = nullptr;
  cudaStream_t s = nullptr;
  int rc = 0;
  std::vector<float4> hf(n);
  std::vector<float> ht(n * 40, 0.0f);
  for (size_t i = 0; i < n; i++) {
    hf[i] = make_float4(feat[3 * i], feat[3 * i + 1], feat[3 * i + 2], 0.0f);
    for (int j = 0; j < NO; j++) ht[i * 40 + j] = target[i * NO + j];
  }
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || N.alloc() ||
      w.alloc(n, true) || cudaMalloc(&df, n * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&dt, n * 40 * sizeof(float)) != cudaSuccess || device_error_flag(&err))
    rc = set_error("kqed_mlp_forward_backward: out of memory");
  if (!rc && (cudaMemcpyAsync(df, hf.data(), n * sizeof(float4), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(dt, ht.data(), n * 40 * sizeof(float), cudaMemcpyHostToDevice, s) ||
              cudaMemsetAsync(err, 0, sizeof(int), s) || upload_params(N, params, s) ||
              forward(N, df, nullptr, n, w, true, err, s) ||
              backward(N, df, dt, (int)n, w, err, s)))
    rc = set_error("kqed_mlp_forward_backward: launch failed");
  std::vector<float> hy(n * NOP), lp(1024);
  const int lb = (int)std::min<size_t>((n + 255) / 256, 1024);
  int herr = 0;
  if (!rc && (cudaMemcpyAsync(hy.data(), w.Y, n * NOP * sizeof(float), cudaMemcpyDeviceToHost, s) ||
              (grad && cudaMemcpyAsync(grad, N.G, kParams * sizeof(float), cudaMemcpyDeviceToHost, s)) ||
              cudaMemcpyAsync(lp.data(), w.lossp, lb * sizeof(float), cudaMemcpyDeviceToHost, s) ||
              cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s) ||
              cudaStreamSynchronize(s)))
    rc = set_error("kqed_mlp_forward_backward: execution failed");
  if (!rc && herr) rc = set_error("kqed_mlp_forward_backward: a tensor-core wait timed out");
  if (!rc) {
    if (y)
      for (size_t i = 0; i < n; i++)
        for (int j = 0; j < NO; j++) y[i * NO + j] = hy[i * NOP + j];
    if (loss) {
      double l = 0.0;
      for (int i = 0; i < lb; i++) l += lp[i];
      *loss = l / ((double)n * NO);
    }
  }
  N.release();
  w.release();
  if (df) cudaFree(df);
  if (dt) cudaFree(dt);
  if (s) cudaStreamDestroy(s);
  return rc;
}

extern "C" size_t kqed_mlp_param_count(void) { return mlp::kParams; }

/* the trained network's parameters and target scaling (host buffers):
   params[kParams]; norm[9 + 3 * 39] = lo[3], sc[3], (unused)[3], oa[39],
   ob[39], os[39] */
extern "C" int kqed_surrogate_export(const struct QED_kernel_temps *t, float *params, float *norm)
{
  if (!t || !t->Grid.PC) return set_error("tables not initialised");
  mlp::Surrogate *S = mlp::find(t->Grid.PC->Fm);
  if (!S) return set_error("no surrogate: train one for these tables first");
  if (params &&
      cudaMemcpy(params, S->net.P, mlp::kParams * sizeof(float), cudaMemcpyDeviceToHost) !=
          cudaSuccess)
    return set_error("kqed_surrogate_export: copy failed");
  if (norm) {
    for (int i = 0; i < 3; i++) {
      norm[i] = S->norm.lo[i];
      norm[3 + i] = S->norm.sc[i];
      norm[6 + i] = 0.0f;
    }
    for (int j = 0; j < mlp::NO; j++) {
      norm[9 + j] = S->norm.oa[j];
      norm[9 + 39 + j] = S->norm.ob[j];
      norm[9 + 78 + j] = S->norm.os[j];
    }
  }
  return 0;
}

/* pairs the network evaluated in lattice sums since the last call (then
   reset); synchronises the device */
extern "C" int kqed_surrogate_served(const struct QED_kernel_temps *t, uint64_t *served)
{
  if (!t || !t->Grid.PC || !served) return set_error("tables not initialised");
  mlp::Surrogate *S = mlp::find(t->Grid.PC->Fm);
  if (!S) return set_error("no surrogate: train one for these tables first");
  *served = 0;
  if (!S->ecount) return 0;
  unsigned long long v = 0;
  if (cudaDeviceSynchronize() != cudaSuccess ||
      cudaMemcpy(&v, S->ecount + 2, sizeof(v), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemset(S->ecount + 2, 0, sizeof(v)) != cudaSuccess)
    return set_error("kqed_surrogate_served: copy failed");
  *served = v;
  return 0;
}

/* The fused evaluation kernel on host data (for checking it): params as
   exported, feat[n][3]; y[n][39] */
extern "C" int kqed_mlp_infer(const float *params, size_t n, const float *feat, float *y)
{
  using namespace mlp;
  if (!params || !feat || !y || n == 0) return set_error("kqed_mlp_infer: bad arguments");
  Net N;
  float4 *df = nullptr;
  float *dy = nullptr;
  int *err = nullptr;
  cudaStream_t s = nullptr;
  int rc = 0;
  std::vector<float4> hf(n);
  for (size_t i = 0; i < n; i++) hf[i] = make_float4(feat[3 * i], feat[3 * i + 1], feat[3 * i + 2], 0.0f);
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || N.alloc() ||
      cudaMalloc(&df, n * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&dy, n * NOP * sizeof(float)) != cudaSuccess || device_error_flag(&err))
    rc = set_error("kqed_mlp_infer: out of memory");
  if (!rc && (cudaMemcpyAsync(df, hf.data(), n * sizeof(float4), cudaMemcpyHostToDevice, s) ||
              cudaMemsetAsync(err, 0, sizeof(int), s) || upload_params(N, params, s) ||
              launch_build_wimg(N.P, N.wimg, s) || infer(N, df, nullptr, n, dy, err, s)))
    rc = set_error("kqed_mlp_infer: launch failed");
  std::vector<float> hy(n * NOP);
  int herr = 0;
  if (!rc && (cudaMemcpyAsync(hy.data(), dy, n * NOP * sizeof(float), cudaMemcpyDeviceToHost, s) ||
              cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s) ||
              cudaStreamSynchronize(s)))
    rc = set_error("kqed_mlp_infer: execution failed");
  if (!rc && herr) rc = set_error("kqed_mlp_infer: a tensor-core wait timed out");
  if (!rc)
    for (size_t i = 0; i < n; i++)
      for (int j = 0; j < NO; j++) y[i * NO + j] = hy[i * NOP + j];
  N.release();
  if (df) cudaFree(df);
  if (dy) cudaFree(dy);
  if (s) cudaStreamDestroy(s);
  return rc;
}
