"""CUDA kernel parity against the oracle and the reference's fixtures, through
the C ABI.  Tolerance: per-pair norm-relative error max_i |d_i| / max_i |ref_i|
<= 1e-12 (plain FP64 form)."""
import ctypes
import os

import numpy as np
import pytest

from _helpers import GOLDEN, norm_rel, oracle_branch, oracle_contract, oracle_kernel

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


def test_config1_L0_matches_oracle(temps):
    """4096 generic pairs in [-2,2]^4 plus 64 with a tiny side"""
    from kqed_gb300.workloads import config1_pairs
    x, y = config1_pairs()
    got, st = K().kernel_batch(temps, 0, x, y, with_status=True)
    ref = oracle_kernel(0, x, y)
    zr = np.abs(ref).max(1) == 0
    assert np.array_equal(zr, np.abs(got).max(1) == 0)
    err = norm_rel(got[~zr], ref[~zr])
    assert err.max() <= TOL, (err.max(), int(np.argmax(err)))
    code = oracle_branch(x, y)
    assert np.array_equal((st & 2) != 0, (code & 7) == 5)   # Taylor-in-x
    assert np.array_equal((st & 4) != 0, (code & 8) != 0)   # swap branch


@pytest.mark.parametrize("variant", [1, 2, 3])
def test_variants_match_oracle(temps, variant):
    rng = np.random.default_rng(10 + variant)
    x = rng.uniform(-2, 2, (768, 4))
    y = rng.uniform(-2, 2, (768, 4))
    x[:16] = 0.0                  # x = 0
    y[16:32] = 0.0                # y = 0
    y[32:48] = x[32:48]           # x = y
    x[48:64] *= 1e-4              # Taylor in x
    got = K().kernel_batch(temps, variant, x, y)
    ref = oracle_kernel(variant, x, y)
    scale = np.maximum(np.abs(ref).max(1), 1e-12 * np.abs(ref).max())
    err = np.abs(got - ref).max(1) / scale
    assert err.max() <= TOL, err.max()


def test_reference_fixtures(temps):
    """outputs of the reference library itself on the synthetic table"""
    fx = np.load(os.path.join(GOLDEN, "ref_synth.npz"))
    for v in range(4):
        got = K().kernel_batch(temps, v, fx["x"], fx["y"])
        ref = fx["L%d" % v]
        nz = np.abs(ref).max(1) > 0
        assert np.array_equal(nz, np.abs(got).max(1) > 0)
        assert norm_rel(got[nz], ref[nz]).max() <= TOL


def test_reference_golden_files(temps):
    fx = np.load(os.path.join(GOLDEN, "reg_axis.npz"))
    got = K().kernel_batch(temps, 0, fx["x"], fx["y"])
    for g, r in zip(got, fx["L0"]):
        assert np.all(np.abs(g - r) <= 5e-6 * np.abs(r) + 1e-6 * np.abs(r).max())


def test_legacy_per_pair_calls(temps):
    """QED_kernel_L0..L3 with the struct passed by value, as a C caller does"""
    rng = np.random.default_rng(5)
    x = rng.uniform(-1.5, 1.5, (6, 4))
    y = rng.uniform(-1.5, 1.5, (6, 4))
    for v in range(4):
        batch = K().kernel_batch(temps, v, x, y)
        for i in range(6):
            one = getattr(K(), "QED_kernel_L%d" % v)(x[i], y[i], temps).reshape(384)
            assert np.array_equal(one, batch[i])


def test_edge_cases(temps):
    g = temps.grid()
    xhi, yhi = g["XX"][-1], g["YY"][-1]
    e = np.array([0.5, 0.5, 0.5, 0.5])
    x = np.array([
        np.zeros(4),                      # x = y = 0 -> zero kernel
        [xhi, 0.0, 0.0, 0.0],             # |x| exactly the last x node (flag_hx edge)
        [xhi * 1.0001, 0.0, 0.0, 0.0],    # beyond the grid -> zero kernel
        e * 0.3,                          # generic partner with |y| beyond the y grid
        e * 2.0,                          # x = y
        [1e-9, 0, 0, 0],                  # tiny but non-zero x
    ])
    y = np.array([
        np.zeros(4),
        [0.1, -0.2, 0.3, 0.05],
        [0.1, -0.2, 0.3, 0.05],
        [yhi * 1.2, 0.0, 0.0, 0.0],
        e * 2.0,
        [0.7, 0.1, -0.3, 0.2],
    ])
    got, st = K().kernel_batch(temps, 0, x, y, with_status=True)
    ref = oracle_kernel(0, x, y)
    assert np.abs(got[0]).max() == 0 and np.abs(got[2]).max() == 0
    assert st[2] & 1
    nz = np.abs(ref).max(1) > 0
    assert np.array_equal(nz, np.abs(got).max(1) > 0)
    assert norm_rel(got[nz], ref[nz]).max() <= TOL


def test_empty_batch(temps):
    out = K().kernel_batch(temps, 2, np.zeros((0, 4)), np.zeros((0, 4)))
    assert out.shape == (0, 384)


def test_parity_identity_large(temps):
    """L^i(x,y) = -L^i(-x,-y) on 65536 pairs (size-independent property)"""
    rng = np.random.default_rng(11)
    x = rng.uniform(-3, 3, (65536, 4))
    y = rng.uniform(-3, 3, (65536, 4))
    a = K().kernel_batch(temps, 0, x, y)
    b = K().kernel_batch(temps, 0, -x, -y)
    assert np.abs(a + b).max() <= 1e-12 * np.abs(a).max()


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_lattice_sum_matches_oracle(temps, variant):
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_numpy
    ys = lattice_sites(6, 0.25)            # 1296 sites
    xs = diagonal_x(4, 0.25)               # includes x = 0
    pi = pi_synth_numpy(xs, ys, seed=3)
    got = K().lattice_sum(temps, variant, xs, ys, pi)
    for k in range(len(xs)):
        X = np.repeat(xs[k:k + 1], len(ys), 0)
        terms = oracle_contract(variant, X, ys, pi[k])
        ref = np.sum(terms)
        scale = np.sum(np.abs(terms))
        assert abs(got[k] - ref) <= TOL * scale, (k, got[k], ref, scale)


def test_lattice_sum_linear_in_pi(temps):
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_numpy
    ys = lattice_sites(4, 0.3)
    xs = diagonal_x(3, 0.3)
    p1 = pi_synth_numpy(xs, ys, seed=4)
    p2 = pi_synth_numpy(xs, ys, seed=5)
    s1 = K().lattice_sum(temps, 2, xs, ys, p1)
    s2 = K().lattice_sum(temps, 2, xs, ys, p2)
    s12 = K().lattice_sum(temps, 2, xs, ys, p1 + 2.0 * p2)
    assert np.allclose(s12, s1 + 2.0 * s2, rtol=1e-12, atol=1e-12 * np.abs(s12).max())


def test_launches_counted(temps):
    n0 = K().launch_count()
    K().kernel_batch(temps, 0, np.ones((4, 4)), np.ones((4, 4)) * 0.5)
    assert K().launch_count() > n0
