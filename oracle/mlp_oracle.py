"""ORACLE -- test infrastructure only.

CPU restatement (numpy, float64) of the learned surrogate's network and of
its training gradient, the checker for the GPU kernels of
kqed_gb300/csrc/kqed_mlp.cu and kqed_mlp_gemm.cu.  The product never calls
it.  It has no counterpart in the reference library (the reference
interpolates its weight functions; the network is this project's addition),
so it is pinned by a finite-difference check of its own gradient
(tests/test_mlp_oracle_cpu.py).

Network: 3 -> 256 -> 256 -> 256 -> 39 (48 padded), SiLU, parameters in one
flat float32 vector in the layout of kqed_mlp.cu:
  W1[256][3] b1[256] W2[256][256] b2[256] W3[256][256] b3[256]
  W4[48][256] b4[48]          (rows 39..47 of W4 and b4 are unused)
Loss: mean over samples and the 39 outputs of (y - t)^2.

With bf16=True the oracle rounds to bfloat16 exactly where the GPU does:
the inputs of every tensor-core product (activations H1..H3, the weight
copies W2..W4, the output gradient dY and the hidden gradients dZ3, dZ2);
layer 1 and all accumulation stay at higher precision.
"""
import numpy as np

H, NIN, NO, NOP = 256, 3, 39, 48
oW1 = 0
ob1 = oW1 + H * NIN
oW2 = ob1 + H
ob2 = oW2 + H * H
oW3 = ob2 + H
ob3 = oW3 + H * H
oW4 = ob3 + H
ob4 = oW4 + NOP * H
NPARAM = ob4 + NOP


def bf16(a):
    """round float64 values to bfloat16 (nearest, ties to even), as float64"""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return {
        "W1": p[oW1:ob1].reshape(H, NIN), "b1": p[ob1:oW2],
        "W2": p[oW2:ob2].reshape(H, H), "b2": p[ob2:oW3],
        "W3": p[oW3:ob3].reshape(H, H), "b3": p[ob3:oW4],
        "W4": p[oW4:ob4].reshape(NOP, H)[:NO], "b4": p[ob4:ob4 + NO],
    }


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, feat, bf=True):
    """outputs [n][39] and the activations the backward pass needs"""
    P = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    f = np.asarray(feat, dtype=np.float64)
    z1 = f @ P["W1"].T + P["b1"]
    h1 = r(silu(z1))
    z2 = h1 @ r(P["W2"]).T + P["b2"]
    h2 = r(silu(z2))
    z3 = h2 @ r(P["W3"]).T + P["b3"]
    h3 = r(silu(z3))
    y = h3 @ r(P["W4"]).T + P["b4"]
    return y, (f, z1, h1, z2, h2, z3, h3)


def loss_and_grad(p, feat, target, bf=True):
    """(loss, gradient [NPARAM], outputs) of the mean-square loss"""
    P = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    y, (f, z1, h1, z2, h2, z3, h3) = forward(p, feat, bf)
    t = np.asarray(target, dtype=np.float64)
    n = len(f)
    d = y - t
    loss = np.mean(d * d)
    dy = 2.0 * d / (n * NO)
    g = np.zeros(NPARAM)
    dyb = r(dy)
    g[oW4:oW4 + NO * H] = (dyb.T @ h3).reshape(-1)
    g[ob4:ob4 + NO] = dy.sum(0)
    dz3 = (dyb @ r(P["W4"])) * dsilu(z3)
    g[ob3:oW4] = dz3.sum(0)
    dz3b = r(dz3)
    g[oW3:ob3] = (dz3b.T @ h2).reshape(-1)
    dz2 = (dz3b @ r(P["W3"])) * dsilu(z2)
    g[ob2:oW3] = dz2.sum(0)
    dz2b = r(dz2)
    g[oW2:ob2] = (dz2b.T @ h1).reshape(-1)
    dz1 = (dz2b @ r(P["W2"])) * dsilu(z1)
    g[ob1:oW2] = dz1.sum(0)
    g[oW1:ob1] = (dz1.T @ f).reshape(-1)
    return loss, g, y


def init_params(seed):
    """He-uniform weights, small random biases (any seeded draw serves the tests)"""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    p[oW1:ob1] = rng.uniform(-1, 1, H * NIN) * np.sqrt(6.0 / NIN)
    p[oW2:ob2] = rng.uniform(-1, 1, H * H) * np.sqrt(6.0 / H)
    p[oW3:ob3] = rng.uniform(-1, 1, H * H) * np.sqrt(6.0 / H)
    p[oW4:oW4 + NO * H] = rng.uniform(-1, 1, NO * H) * np.sqrt(1.0 / H)
    p[ob1:oW2] = rng.uniform(-0.1, 0.1, H)
    p[ob2:oW3] = rng.uniform(-0.1, 0.1, H)
    p[ob3:oW4] = rng.uniform(-0.1, 0.1, H)
    p[ob4:ob4 + NO] = rng.uniform(-0.1, 0.1, NO)
    return p


BLOCKS = {"W1": (oW1, ob1), "b1": (ob1, oW2), "W2": (oW2, ob2), "b2": (ob2, oW3),
          "W3": (oW3, ob3), "b3": (ob3, oW4), "W4": (oW4, oW4 + NO * H), "b4": (ob4, ob4 + NO)}
