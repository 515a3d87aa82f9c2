"""The mixed-precision form (KQED_FP32_MIXED) against the oracle and the FP64
form, through the C ABI.

Tolerances, written here and in the assertions:
  * per pair, norm-relative max_i |d_i| / max_i |ref_i| <= 2e-5, median
    <= 1e-6 (float interpolation and assembly, FP64 invariants, chain rule
    and sums);
  * pairs the mixed form assembles in FP64 (x = 0, y = 0, x = y,
    |x - y| < max(|x|, |y|) / 4 and max(|x|, |y|) < 0.35) equal the FP64
    form to 1e-13 per pair (the same FP64 code, compiled into a different
    kernel, may contract a*b + c*d into FMAs differently);
  * fused lattice sums: per x, |S_mixed - S_fp64| <= 1e-6 * rms_x(S_fp64),
    the integrand error the mixed form is built to meet.
"""
import numpy as np
import pytest

from _helpers import norm_rel, oracle_kernel

pytestmark = pytest.mark.gpu

PAIR_MAX = 2e-5
PAIR_MEDIAN = 1e-6
SUM_TOL = 1e-6
ROUTED_TOL = 1e-13


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


def test_mixed_config1_L0_against_oracle(temps):
    from kqed_gb300.workloads import config1_pairs
    x, y = config1_pairs()
    got = K().kernel_batch(temps, 0, x, y, precision=K().KQED_FP32_MIXED)
    ref = oracle_kernel(0, x, y)
    zr = np.abs(ref).max(1) == 0
    assert np.array_equal(zr, np.abs(got).max(1) == 0)
    err = norm_rel(got[~zr], ref[~zr])
    assert err.max() <= PAIR_MAX, (err.max(), int(np.argmax(err)))
    assert np.median(err) <= PAIR_MEDIAN, np.median(err)


@pytest.mark.parametrize("variant", [1, 2, 3])
def test_mixed_variants_against_oracle(temps, variant):
    rng = np.random.default_rng(40 + variant)
    x = rng.uniform(-2, 2, (512, 4))
    y = rng.uniform(-2, 2, (512, 4))
    x[:16] = 0.0
    y[16:32] = 0.0
    y[32:48] = x[32:48]
    x[48:64] *= 1e-4
    got = K().kernel_batch(temps, variant, x, y, precision=K().KQED_FP32_MIXED)
    ref = oracle_kernel(variant, x, y)
    scale = np.maximum(np.abs(ref).max(1), 1e-12 * np.abs(ref).max())
    err = np.abs(got - ref).max(1) / scale
    assert err.max() <= PAIR_MAX, (err.max(), int(np.argmax(err)))


def test_mixed_fp64_routed_pairs_are_exact(temps):
    """x = 0, y = 0, x = y and near pairs are assembled in FP64"""
    rng = np.random.default_rng(77)
    x = rng.uniform(-2, 2, (256, 4))
    # |x - y| <= 0.1 |x|
    y = x + 0.05 * np.linalg.norm(x, axis=1)[:, None] * rng.uniform(-1, 1, (256, 4))
    x[:32] = 0.0
    y[32:64] = 0.0
    y[64:96] = x[64:96]
    d = np.linalg.norm(x - y, axis=1)
    big = np.maximum(np.linalg.norm(x, axis=1), np.linalg.norm(y, axis=1))
    routed = (d ** 2 * 16 < big ** 2) | (d == 0) | (np.abs(x).max(1) == 0) | (np.abs(y).max(1) == 0)
    assert routed.all()
    a = K().kernel_batch(temps, 0, x, y, precision=K().KQED_FP64)
    b = K().kernel_batch(temps, 0, x, y, precision=K().KQED_FP32_MIXED)
    err = norm_rel(b, a)
    assert err.max() <= ROUTED_TOL, err.max()


@pytest.mark.parametrize("variant", [0, 2, 3])
def test_mixed_lattice_sum_within_integrand_tolerance(temps, variant):
    import torch
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_torch
    ys = lattice_sites(12, 0.15)
    rng = np.random.default_rng(5)
    xs = np.vstack([diagonal_x(9, 0.3)[1:], rng.uniform(-1.2, 1.2, (8, 4))])
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    pi = pi_synth_torch(xs, ys, seed=11, device="cuda")
    out = {}
    for p in (K().KQED_FP64, K().KQED_FP32_MIXED):
        s = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
        K().lattice_sum_dev(temps, variant, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys),
                            pi.data_ptr(), s.data_ptr(), p)
        torch.cuda.synchronize()
        out[p] = s.cpu().numpy()
    a, b = out[K().KQED_FP64], out[K().KQED_FP32_MIXED]
    rms = np.sqrt(np.mean(a ** 2))
    err = np.abs(b - a) / rms
    assert err.max() <= SUM_TOL, (err.max(), xs[int(np.argmax(err))])


def test_mixed_lattice_host_entry_matches_device_entry(temps):
    """kqed_lattice_sum (host buffers, chunked copies) gives the device
    entry point's result in the mixed form too"""
    import torch
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_torch
    ys = lattice_sites(8, 0.2)
    xs = diagonal_x(5, 0.2)
    pi = pi_synth_torch(xs, ys, seed=3, device="cuda")
    s = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    K().lattice_sum_dev(temps, 2, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), pi.data_ptr(),
                        s.data_ptr(), K().KQED_FP32_MIXED)
    torch.cuda.synchronize()
    host = K().lattice_sum(temps, 2, xs, ys, pi.cpu().numpy(), precision=K().KQED_FP32_MIXED)
    assert np.array_equal(host, s.cpu().numpy())


def test_precision_stats_match_host_statistics(temps):
    """kqed_precision_stats accumulates on the device what the host computes
    from the two forms' batch outputs (L3, pairs as in the 1e8-pair
    statistics workload: U[-4,4]^4 with 1% small |x| or |y|)"""
    import torch
    rng = np.random.default_rng(4)
    n = 3000
    x = rng.uniform(-4, 4, (n, 4))
    y = rng.uniform(-4, 4, (n, 4))
    small = rng.random(n) < 0.01
    x[small[: n // 2].nonzero()[0]] *= 1e-3
    y[n // 2:][small[n // 2:]] *= 1e-3
    a = K().kernel_batch(temps, 3, x, y, precision=K().KQED_FP64)
    b = K().kernel_batch(temps, 3, x, y, precision=K().KQED_FP32_MIXED)
    floor = 1e-30
    nrm = np.abs(a).max(1)
    live = (nrm > 0) | (np.abs(b).max(1) > 0)
    r = np.abs(b - a)[live] / np.maximum(nrm[live], floor)[:, None]
    dx = torch.as_tensor(x, device="cuda")
    dy = torch.as_tensor(y, device="cuda")
    st = K().precision_stats(temps, 3, dx.data_ptr(), dy.data_ptr(), n, floor)
    assert st["pairs"] == int(live.sum())
    np.testing.assert_allclose(st["comp_max"], r.max(0), rtol=1e-12, atol=0)
    np.testing.assert_allclose(st["comp_rms"], np.sqrt((r ** 2).mean(0)), rtol=1e-9, atol=0)
    assert abs(st["pair_max"] - r.max()) <= 1e-12 * r.max()
    assert abs(st["pair_mean"] - r.max(1).mean()) <= 1e-9 * r.max(1).mean()
    assert st["pair_max"] <= PAIR_MAX
