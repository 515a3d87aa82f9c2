"""The oracle's restatement of the reference's composite kernels
(all_kernels.c, con_kernel.c, sub_kernel.c, SYMXY.c, SYMXY0.c,
kernels.c:181-231), pinned to the reference library's own outputs (the
committed fixture and, where the reference was built here, the live
library), and the reference's identity tests run on it.  CPU only.

Tolerance: |oracle - reference| <= 1e-13 * scale per pair, scale = the
largest |L0| the composite combines; the composites' outputs can be orders
of magnitude below their terms (|x| near zero makes L0(y, x) large), so the
output's own magnitude is not the scale of its rounding."""
import ctypes
import os

import numpy as np
import pytest

import _composite_checks as C
from _helpers import (COMPOSITE_SIZE, COMPOSITES, GOLDEN, PKG, REF_SO, composite_masses,
                      composite_pairs, composite_scale, oracle_composite, oracle_kernel)

TOL = 1e-13


def test_composite_sizes_are_the_reference_structs():
    sizes = {"QED_Kernels": 8 * 384, "Kernels": 4 * 384, "Kernels3": 12 * 384, "kernel": 384}
    want = ["QED_Kernels"] * 4 + ["Kernels3"] * 3 + ["QED_Kernels", "Kernels", "QED_Kernels",
                                                     "Kernels", "kernel"]
    assert COMPOSITE_SIZE == [sizes[w] for w in want]


@pytest.mark.parametrize("which", range(12), ids=COMPOSITES)
def test_oracle_composite_matches_reference_fixture(which):
    fx = np.load(os.path.join(GOLDEN, "ref_composite.npz"))
    x, y, ref, scale = (fx["%s%d" % (k, which)] for k in ("x", "y", "out", "scale"))
    got = oracle_composite(which, x, y, composite_masses(which))
    d = np.abs(got - ref).max(1)
    assert np.all(d <= TOL * scale), d / scale


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")
def test_oracle_composites_match_live_reference():
    os.environ["KQEDREF_PATH"] = PKG
    L = ctypes.CDLL(REF_SO)
    assert L.ref_init() == 0
    dp = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(31)
    px, py = composite_pairs()
    x = np.vstack([px, rng.uniform(-2, 2, (24, 4))])
    y = np.vstack([py, rng.uniform(-2, 2, (24, 4))])
    for which in range(12):
        M = composite_masses(which)
        got = oracle_composite(which, x, y, M)
        ref = np.zeros_like(got)
        assert L.ref_composite(which, M.ctypes.data_as(dp), len(x), x.ctypes.data_as(dp),
                               y.ctypes.data_as(dp), ref.ctypes.data_as(dp), 0) == 0
        scale = composite_scale(which, x, y)
        d = np.abs(got - ref).max(1)
        assert np.all(d <= TOL * scale), (COMPOSITES[which], (d / scale).max())


def test_reference_identities_on_the_oracle():
    """src/amu_forlattice.c examples 12-21 and 23 on the oracle"""
    px, py = composite_pairs()
    sel = [0, 1, 2, 5, 6]      # generic, swap, tiny x, x = y, same ray
    x, y = px[sel], py[sel]
    comp = lambda w, a, b, M: oracle_composite(w, a, b, M)
    C.run_all(comp, oracle_kernel, x, y, lambda a, b: oracle_kernel(0, a, b))


def test_swap_and_average_helpers():
    """swap_munu_Lyx (all_kernels.c:373-406; example 19, src/amu_forlattice.c:1015-1078)
    and the average_* helpers of the library, host code only"""
    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300 as K
    L = K.lib()
    rng = np.random.default_rng(2)
    q = rng.standard_normal(3072)
    a = q.copy()
    L.swap_munu_Lyx(a.ctypes.data_as(ctypes.c_void_p))
    Q, A = C.qk(q[None]), C.qk(a[None])
    assert np.array_equal(A[:, :, 0], Q[:, :, 0])
    assert np.array_equal(A[:, :, 1], C.perm(Q[:, :, 1], "kjl"))
    for name, n, byval in (("average_all_kernels", 1536, True),
                           ("average_all_QED_kernels", 3072, True),
                           ("average_con_kernels", 4608, False)):
        k = rng.standard_normal(n)
        w = rng.standard_normal(n)
        want = 0.5 * (k + w)
        f = getattr(L, name)
        if byval:
            class ByValue(ctypes.Structure):   # the struct passed by value
                _fields_ = [("v", ctypes.c_double * n)]
            f.argtypes = [ctypes.c_void_p, ByValue]
            f(k.ctypes.data_as(ctypes.c_void_p), ByValue((ctypes.c_double * n)(*w)))
        else:
            f.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            f(k.ctypes.data_as(ctypes.c_void_p), w.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(k, want), name
