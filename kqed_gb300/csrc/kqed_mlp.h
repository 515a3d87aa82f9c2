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

int gemm_smem_bytes();
/* the calling device's timeout flag for the tensor-core kernels */
int device_error_flag(int **out);
/* splits > 1 (mode STORE only): K split across blockIdx.z, one partial each */
cudaError_t launch_gemm(const GemmArgs &g, int splits, cudaStream_t s);

} // namespace mlp
} // namespace kqed

#endif
