"""The composite kernels on the GPU (kqed_composite_batch and the
reference-signature calls), checked against the oracle, the reference
library's own outputs (committed fixture) and the reference's identity
tests (src/amu_forlattice.c examples 12-21, 23).

Tolerance: FP64 form, |gpu - oracle| <= 1e-12 * scale per pair, scale =
the largest |L0| the composite combines (an output can be far smaller than
its terms; the reference's own tests use an absolute 1e-12 on kernels of
order one).  Mixed form: <= 2e-5 * scale."""
import os

import numpy as np
import pytest

import _composite_checks as C
from _helpers import (COMPOSITE_SIZE, COMPOSITES, GOLDEN, composite_masses, composite_pairs,
                      composite_scale, oracle_composite, oracle_kernel)

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


def _pairs():
    """seeded random pairs plus the branch-covering ones, in the grid"""
    rng = np.random.default_rng(99)
    px, py = composite_pairs()
    x = np.vstack([px, rng.uniform(-2, 2, (40, 4)), 1e-3 * rng.uniform(-1, 1, (4, 4))])
    y = np.vstack([py, rng.uniform(-2, 2, (40, 4)), rng.uniform(-1, 1, (4, 4))])
    return x, y


@pytest.mark.parametrize("which", range(12), ids=COMPOSITES)
def test_composite_matches_oracle(temps, which):
    x, y = _pairs()
    M = composite_masses(which)
    got = K().composite_batch(temps, which, x, y, M)
    ref = oracle_composite(which, x, y, M)
    scale = composite_scale(which, x, y)
    d = np.abs(got - ref).max(1)
    assert got.shape == (len(x), COMPOSITE_SIZE[which])
    assert np.all(d <= TOL * scale), ((d / scale).max(), int(np.argmax(d / scale)))


@pytest.mark.parametrize("which", range(12), ids=COMPOSITES)
def test_composite_matches_reference_fixture(temps, which):
    fx = np.load(os.path.join(GOLDEN, "ref_composite.npz"))
    x, y, ref, scale = (fx["%s%d" % (k, which)] for k in ("x", "y", "out", "scale"))
    got = K().composite_batch(temps, which, x, y, composite_masses(which))
    d = np.abs(got - ref).max(1)
    assert np.all(d <= TOL * scale), d / scale


def test_reference_signature_calls_equal_the_batch(temps):
    """compute_con_kernelsM_L2(M, x, y, t, K) etc. through the C ABI, one pair
    each, give the batch's bits"""
    px, py = composite_pairs()
    for which, name in enumerate(K().COMPOSITE_FUNCS + ["QED_Mkernel_L2"]):
        M = composite_masses(which)
        batch = K().composite_batch(temps, which, px[:2], py[:2], M)
        for i in range(2):
            one = K().composite_call(name, px[i], py[i], temps,
                                     M[0] if name == "QED_Mkernel_L2" else M)
            assert np.array_equal(one, batch[i]), (name, i)


def test_reference_identities_on_the_gpu(temps):
    px, py = composite_pairs()
    sel = [0, 1, 2, 5, 6]
    x, y = px[sel], py[sel]
    comp = lambda w, a, b, M: K().composite_batch(temps, w, a, b, M)
    kern = lambda v, a, b: K().kernel_batch(temps, v, a, b)
    C.run_all(comp, kern, x, y, lambda a, b: oracle_kernel(0, a, b))


def test_mixed_form_close_to_fp64(temps):
    x, y = _pairs()
    for which in (K().KQED_MKERNEL_L2, 5, 9):
        M = composite_masses(which)
        a = K().composite_batch(temps, which, x, y, M)
        b = K().composite_batch(temps, which, x, y, M, precision=K().KQED_FP32_MIXED)
        scale = composite_scale(which, x, y)
        d = np.abs(a - b).max(1)
        assert np.all(d <= 2e-5 * scale), (which, (d / scale).max())


def test_batches_across_the_launch_group_boundary(temps):
    """more pairs than one launch group (32768): the pairs after the
    boundary give the same bits as a batch of their own"""
    rng = np.random.default_rng(5)
    n = 32768 + 40
    x = rng.uniform(-2, 2, (n, 4))
    y = rng.uniform(-2, 2, (n, 4))
    which = K().KQED_MKERNEL_L2
    big = K().composite_batch(temps, which, x, y, [0.7])
    tail = K().composite_batch(temps, which, x[-60:], y[-60:], [0.7])
    assert np.array_equal(big[-60:], tail)


def test_errors_and_empty_batches(temps):
    x, y = composite_pairs()
    assert K().composite_batch(temps, 0, x[:0], y[:0]).shape == (0, 3072)
    with pytest.raises(K().KQEDError, match="masses"):
        K().composite_batch(temps, 5, x[:1], y[:1], None)
    with pytest.raises(K().KQEDError, match="unknown composite"):
        K().composite_batch(temps, 12, x[:1], y[:1])
    with pytest.raises(K().KQEDError, match="precision"):
        K().composite_batch(temps, 0, x[:1], y[:1], precision=K().KQED_SURROGATE)
