/*
 * Internal interface of the learned weight-function surrogate: the BF16
 * tensor-core GEMM (kqed_mlp_gemm.cu) and the network's training and
 * evaluation (kqed_mlp.cu).  Not installed; the public ABI is include/kqed.h.
 */
#ifndef KQED_MLP_H
#define KQED_MLP_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace kqed {
namespace mlp {

enum GemmMode { kStore = 0, kHidden = 1, kOut = 2, kBwd = 3 };

/* C = epilogue(A B^T) with A(m, k) = A[m sAm + k sAk], B(n, k) = B[n sBn + k sBk] */
struct GemmArgs {
  const __nv_bfloat16 *A;
  long long sAm, sAk;
  const __nv_bfloat16 *B;
  long long sBn, sBk;
  int M, N, K;
  int mode;
  const float *bias;    /* [N] or NULL (HIDDEN, OUT) */
  const float *zin;     /* [M][ldc] pre-activations (BWD) */
  float *cf;            /* fp32 output [M][ldc] (STORE: [splits][pstride]) */
  long long ldc, pstride;
  __nv_bfloat16 *cb;    /* bf16 output [M][ldb] (HIDDEN, BWD) */
  long long ldb;
  int *err;             /* set to 1 when a bounded wait ran out */
  const unsigned *Mdev; /* if set, the rows are min(M, *Mdev) (a count made on the device) */
  /* set by launch_gemm */
  int bn, ksplit;
};

/* the network: 3 -> 256 -> 256 -> 256 -> 39 (48 on the tensor cores), SiLU;
   parameters in one fp32 vector */
constexpr int kH = 256, kNin = 3, kNo = 39, kNop = 48;
constexpr size_t kOW1 = 0, kOB1 = kOW1 + (size_t)kH * kNin, kOW2 = kOB1 + kH,
                 kOB2 = kOW2 + (size_t)kH * kH, kOW3 = kOB2 + kH, kOB3 = kOW3 + (size_t)kH * kH,
                 kOW4 = kOB3 + kH, kOB4 = kOW4 + (size_t)kNop * kH, kParamCount = kOB4 + kNop;

/* Weight image of the fused evaluation kernel: W2 and W3 each as four
   32 KB chunks of 64 output rows x 256 inputs, then W4 (48 rows, 24 KB),
   every chunk already in the tensor cores' K-major core-matrix layout so
   that one bulk copy moves it into shared memory. */
constexpr size_t kWimgChunk = (size_t)64 * kH * 2;
constexpr size_t kWimgW4 = (size_t)kNop * kH * 2;
constexpr size_t kWimgBytes = 8 * kWimgChunk + kWimgW4;
cudaError_t launch_build_wimg(const float *P, __nv_bfloat16 *wimg, cudaStream_t s);

/* Y[r][48] = net(feat[r]) for r < min(rows, *count) (count NULL: rows), one
   fused persistent kernel: layer 1 on the CUDA cores, layers 2-4 on the
   tensor cores from the weight image, activations kept in shared memory */
struct InferArgs {
  const float4 *feat;
  const unsigned *count;
  size_t rows;
  const float *P;
  const __nv_bfloat16 *wimg;
  float *Y;
  int *err;
};
cudaError_t launch_mlp_infer(const InferArgs &a, cudaStream_t s);

int gemm_smem_bytes();
/* the calling device's timeout flag for the tensor-core kernels */
int device_error_flag(int **out);
/* splits > 1 (mode STORE only): K split across blockIdx.z, one partial each */
cudaError_t launch_gemm(const GemmArgs &g, int splits, cudaStream_t s);

} // namespace mlp
} // namespace kqed

#endif
