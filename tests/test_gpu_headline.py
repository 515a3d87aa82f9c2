"""Parity of the benchmarked workload's geometry and of the grid-edge pairs
against the oracle, through the C ABI (plain FP64 form).

The benchmark sums kernel L2 over the periodic 24^4 lattice at spacing 0.1
for x on the (1,1,1,1) diagonal up to |x| = 6.2, near the top of the x grid
(last node 6.54), where the Chebyshev sums are longest.  Here a slab of
4096 of its sites (every 81st) plus hand-placed sites is summed against x at
k = 0, 8, 31 and one x beyond the grid, for L0..L3.

Grid-edge pairs: the GPU takes every branch and grid decision (zero and
axis tests, |x| beyond the last node, grid search, x <-> (x-y) swap test) on
norms and dot products rounded after every operation, as the reference's
portable build and the oracle compute them (src/HEADERS/getff-new.h:49-53,
src/LIBFILES/getff-new.c:316-370, src/LIBFILES/kernels.c:14-26).  So a pair
whose |x| lies within an ulp of the last x node, or whose |y| equals the
last y node, is decided exactly as the oracle decides it: the zero / nonzero
pattern must match exactly and the values to 1e-12.

Tolerance: lattice sums |S_gpu - S_oracle| <= 1e-12 * sum_y |L.Pi|; pairs
max_c |dL_c| <= 1e-12 * max_c |L_c|."""
import numpy as np
import pytest

from _helpers import norm_rel, oracle_contract, oracle_kernel

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


def headline_slab(grid):
    from kqed_gb300.workloads import lattice_sites
    a = 0.1
    ys = lattice_sites(24, a)[::81]            # 4096 of the 331,776 sites
    d = np.ones(4)
    yhi = grid["YY"][-1]
    extra = np.array([
        0.3 * d, -0.5 * d, 1.1 * d, -1.2 * d,   # on the x diagonal: cb = +-1 exactly
        2.0 * d, -0.05 * d,
        [yhi, 0.0, 0.0, 0.0],                   # |y| at the last y node
        0.5 * yhi * d,                          # |y| = last y node along the diagonal
        [0.0, 0.0, 0.0, -yhi],
    ])
    return np.ascontiguousarray(np.vstack([ys, extra]))


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_headline_geometry_lattice_sum_matches_oracle(temps, variant):
    from kqed_gb300.workloads import pi_synth_numpy
    g = temps.grid()
    a = 0.1
    xs = np.outer(np.array([0.0, 8.0, 31.0, 33.0]) * a, np.ones(4))
    assert np.linalg.norm(xs[3]) > g["XX"][-1] > np.linalg.norm(xs[2])
    ys = headline_slab(g)
    pi = pi_synth_numpy(xs, ys, seed=70 + variant)
    got = K().lattice_sum(temps, variant, xs, ys, pi)
    for k in range(len(xs)):
        X = np.repeat(xs[k:k + 1], len(ys), 0)
        terms = oracle_contract(variant, X, ys, pi[k])
        ref = np.sum(terms)
        scale = np.sum(np.abs(terms))
        assert abs(got[k] - ref) <= TOL * scale + 1e-300, (variant, k, got[k], ref, scale)


def ulp_edge_pairs(grid):
    """x within 2 ulp of the last x node (on an axis and along the diagonal,
    where |x| itself rounds), against generic partners, partners at the last
    y node, and partners on the same ray (cb = +-1 exactly)."""
    xhi, yhi = grid["XX"][-1], grid["YY"][-1]
    xs, ys = [], []
    rng = np.random.default_rng(77)
    partners = [rng.uniform(-1.5, 1.5, 4) for _ in range(3)]
    for steps in range(-2, 3):
        v = xhi
        for _ in range(abs(steps)):
            v = np.nextafter(v, np.inf if steps > 0 else -np.inf)
        for xv in (np.array([v, 0.0, 0.0, 0.0]), np.full(4, 0.5 * v),
                   np.array([0.0, 0.0, -v, 0.0])):
            for yv in partners + [np.array([0.0, yhi, 0.0, 0.0]), 0.25 * xv, -0.7 * xv]:
                xs.append(xv)
                ys.append(yv)
    return np.array(xs), np.array(ys)


@pytest.mark.parametrize("variant", [0, 2])
def test_ulp_edge_pairs_decided_as_the_oracle_decides(temps, variant):
    g = temps.grid()
    x, y = ulp_edge_pairs(g)
    got = K().kernel_batch(temps, variant, x, y)
    ref = oracle_kernel(variant, x, y)
    zr = np.abs(ref).max(1) == 0
    zg = np.abs(got).max(1) == 0
    assert np.array_equal(zr, zg), np.nonzero(zr != zg)[0]
    # both sides of the boundary occur: some pairs in the grid, some out of it
    if variant == 0:
        assert zr.any() and (~zr).any()
    err = norm_rel(got[~zr], ref[~zr])
    assert err.max() <= TOL, (err.max(), int(np.argmax(err)))


def test_pairs_on_a_ray_off_the_diagonal(temps):
    """cb = +-1 exactly with x != y (y a multiple of x): the Chebyshev sums at
    the ends of [-1, 1], kept in FP64"""
    rng = np.random.default_rng(78)
    x = rng.uniform(-2.0, 2.0, (64, 4))
    s = np.concatenate([rng.uniform(0.1, 0.9, 32), -rng.uniform(0.1, 1.5, 32)])
    y = x * s[:, None]
    for v in range(4):
        got = K().kernel_batch(temps, v, x, y)
        ref = oracle_kernel(v, x, y)
        nz = np.abs(ref).max(1) > 0
        assert np.array_equal(nz, np.abs(got).max(1) > 0)
        assert norm_rel(got[nz], ref[nz]).max() <= TOL
