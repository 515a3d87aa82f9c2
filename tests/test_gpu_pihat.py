"""The perturbative lepton-loop Pi-hat on the GPU (kqed_pihat_batch[_dev],
kqed_pihat_lattice_dev, and ipihatFermLoop_antisym / pihat1 with the
reference's signatures) against the oracle and the reference library's
outputs; and the reference's lepton-loop check of a_mu
(src/amu_forlattice.c:65-116): the integrand L0(x,y) . Pi-hat(2x, 2y) on the
GPU against the oracle's.

Tolerance: 1e-12 of each pair's largest |component| (the kernel keeps the
reference's order of operations; CUDA's exp, log, sqrt differ from libm's by
an ulp)."""
import os

import numpy as np
import pytest

from _helpers import GOLDEN, oracle_contract, oracle_kernel, oracle_pihat

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def temps():
    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300 as K
    t = K.KernelTemps()
    yield t
    t.free()


def K():
    import kqed_gb300
    return kqed_gb300


def close(got, ref):
    scale = np.abs(ref).max(1)
    d = np.abs(got - ref).max(1)
    assert np.all(d <= TOL * scale), (d / scale).max()


def test_pihat_matches_oracle(temps):
    rng = np.random.default_rng(12)
    x = rng.uniform(-2, 2, (96, 4))
    y = rng.uniform(-2, 2, (96, 4))
    x[:8] *= 0.01
    close(K().pihat_batch(x, y), oracle_pihat(x, y))


def test_pihat_matches_reference_fixture(temps):
    fx = np.load(os.path.join(GOLDEN, "ref_pihat.npz"))
    close(K().pihat_batch(fx["x"], fx["y"]), fx["pihat"])
    for i in range(2):
        p, r = K().pihat1(fx["x"][i], fx["y"][i], temps)
        close(np.concatenate([p.ravel(), r.ravel()])[None], fx["pihat1"][i][None])


def test_reference_signature_equals_batch(temps):
    fx = np.load(os.path.join(GOLDEN, "ref_pihat.npz"))
    b = K().pihat_batch(fx["x"][:3], fx["y"][:3])
    for i in range(3):
        one = K().ipihatFermLoop_antisym(fx["x"][i], fx["y"][i], temps)
        assert np.array_equal(one.ravel(), b[i])


def test_lattice_layout(temps):
    import torch
    rng = np.random.default_rng(3)
    xs = rng.uniform(-1, 1, (3, 4))
    ys = rng.uniform(-1, 1, (70, 4))
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    pi = torch.empty((3, 70, 384), dtype=torch.float64, device="cuda")
    K().pihat_lattice_dev(dx.data_ptr(), 3, dy.data_ptr(), 70, 2.0, pi.data_ptr())
    torch.cuda.synchronize()
    X = np.repeat(2.0 * xs, 70, 0)
    Y = np.tile(2.0 * ys, (3, 1))
    assert np.array_equal(pi.cpu().numpy().reshape(-1, 384), K().pihat_batch(X, Y))


def test_lepton_loop_integrand(temps):
    """src/amu_forlattice.c:65-116: for |x|, beta, |y| on the reference's
    grid, 2 |x|^3 |y|^4 sin^2(beta) fnorm sum_c L0_c(x, y) Pi-hat_c(Mv x, Mv y),
    Mv = 2: the GPU's L0 and Pi-hat against the oracle's"""
    Mv = 2.0
    alpha = 1.0 / 137.035999
    pref = ((4.0 * np.pi * alpha) ** 3 / 3) * (2.0 * np.pi ** 2) * (4 * np.pi)
    fnorm = 2.0 * pref * Mv ** 7
    pts = [(a, b, c) for a in np.arange(0.005, 1, 0.2) for b in np.arange(0.005, np.pi, np.pi / 4)
           for c in np.arange(0.005, 1, 0.2)]
    xv = np.array([[0, 0, a * np.sin(b), a * np.cos(b)] for a, b, c in pts])
    yv = np.array([[0, 0, 0, c] for a, b, c in pts])
    w = np.array([2 * a ** 3 * c ** 4 * np.sin(b) ** 2 for a, b, c in pts]) * fnorm
    L = K().kernel_batch(temps, 0, xv, yv)
    P = K().pihat_batch(Mv * xv, Mv * yv)
    got = w * np.einsum("ij,ij->i", L, P)
    Lo = oracle_kernel(0, xv, yv)
    Po = oracle_pihat(Mv * xv, Mv * yv)
    close(P, Po)
    ref = w * oracle_contract(0, xv, yv, Po)
    scale = np.abs(w) * np.einsum("ij,ij->i", np.abs(Lo), np.abs(Po))
    # the grid's first points have x close to y (|x - y| = 5e-3 |x|), where L0's
    # swap branch amplifies last-bit differences (the reference's own AVX and
    # portable builds differ by ~1e-11 there): 1e-9 for |x - y| < |x| / 10
    d = np.linalg.norm(xv - yv, axis=1) / np.maximum(np.linalg.norm(xv, axis=1),
                                                     np.linalg.norm(yv, axis=1))
    tol = np.where(d < 0.1, 1e-9, 1e-12)
    assert np.all(np.abs(got - ref) <= tol * scale + 1e-300)
