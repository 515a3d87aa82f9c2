"""The learned weight-function surrogate on the tensor cores.

BF16 GEMM (tcgen05.mma, FP32 accumulation in tensor memory) through the C
ABI against a float64 product of the same bf16 values: every operand
orientation the network's training uses (X W^T, dZ W, dZ^T H), ragged sizes,
split K.  Tolerance: |C - C_ref| <= 1e-5 * sum_k |A B| + 1e-30 (FP32
accumulation of exact bf16 products)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def K():
    import kqed_gb300
    return kqed_gb300


@pytest.fixture(scope="module")
def built():
    from kqed_gb300 import build as B
    B.build()
    return True


def _bf16(torch, shape, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(shape, generator=g, dtype=torch.float32).to(torch.bfloat16)


@pytest.mark.parametrize("M,N,Kd,ta,tb,splits", [
    (128, 256, 64, False, False, 1),
    (300, 200, 100, False, False, 1),
    (257, 48, 256, False, True, 1),
    (256, 256, 1000, True, True, 4),
    (64, 16, 8, False, False, 1),
    (520, 256, 256, False, False, 1),
])
def test_bf16_gemm_matches_float64(built, M, N, Kd, ta, tb, splits):
    import torch
    a = _bf16(torch, (Kd, M) if ta else (M, Kd), 1 + M)
    b = _bf16(torch, (Kd, N) if tb else (N, Kd), 2 + N)
    da, db = a.cuda(), b.cuda()
    c = torch.full((splits, M, N), float("nan"), dtype=torch.float32, device="cuda")
    sam, sak = (1, M) if ta else (Kd, 1)
    sbn, sbk = (1, N) if tb else (Kd, 1)
    K().bf16_gemm(da.data_ptr(), sam, sak, db.data_ptr(), sbn, sbk, M, N, Kd, c.data_ptr(), N,
                  splits=splits)
    A = (a.T if ta else a).double().numpy()
    B = (b.T if tb else b).double().numpy()
    ref = A @ B.T
    scale = np.abs(A) @ np.abs(B).T
    got = c.double().sum(0).cpu().numpy()
    assert np.all(np.isfinite(got))
    err = np.abs(got - ref) / (scale + 1e-30)
    assert err.max() <= 1e-5, (err.max(), np.unravel_index(np.argmax(err), err.shape))
