"""The perturbative lepton-loop Pi-hat (the reference's
src/LIBFILES/pi_pert.c): the oracle's restatement pinned to the reference
library's outputs (fixture, and the live library where it was built here),
and the library's host functions of the same file (init_g8, diractrace,
bessk, amu_heavlept, amu_lightlept, vac_pol) against the reference's
values.  CPU only: no kernel runs.

Tolerances: Pi-hat 1e-13 of the pair's largest |component| (the oracle
keeps the reference's order of operations; observed exact); the analytic
functions 1e-14 relative; G8 and the traces exact."""
import ctypes
import os

import numpy as np
import pytest

from _helpers import GOLDEN, PKG, REF_SO, oracle_g8, oracle_pihat

FIX = os.path.join(GOLDEN, "ref_pihat.npz")


@pytest.fixture(scope="module")
def lib():
    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300 as K
    L = K.lib()
    for f in ("amu_heavlept", "amu_lightlept", "vac_pol"):
        getattr(L, f).restype = ctypes.c_double
        getattr(L, f).argtypes = [ctypes.c_double]
    L.bessk.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    L.diractrace.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    return L


def test_oracle_pihat_matches_reference_fixture():
    fx = np.load(FIX)
    got = oracle_pihat(fx["x"], fx["y"])
    ref = fx["pihat"]
    scale = np.abs(ref).max(1)
    assert np.all(np.abs(got - ref).max(1) <= 1e-13 * scale)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")
def test_oracle_pihat_and_g8_match_live_reference():
    os.environ["KQEDREF_PATH"] = PKG
    L = ctypes.CDLL(REF_SO)
    assert L.ref_init() == 0
    g = np.zeros(65536, dtype=np.int32)
    assert L.ref_g8(g.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 0
    assert np.array_equal(g, oracle_g8())
    dp = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(41)
    x = rng.uniform(-2, 2, (32, 4))
    y = rng.uniform(-2, 2, (32, 4))
    ref = np.zeros((32, 384))
    L.ref_pihat(32, x.ctypes.data_as(dp), y.ctypes.data_as(dp), ref.ctypes.data_as(dp), 0)
    got = oracle_pihat(x, y)
    assert np.all(np.abs(got - ref).max(1) <= 1e-13 * np.abs(ref).max(1))


def test_library_g8_and_traces(lib):
    """init_g8 fills the table as the reference's initialise does; diractrace
    of short products by the Clifford algebra"""
    import kqed_gb300 as K
    t = K.QED_kernel_temps()
    buf = (ctypes.c_int * 65536)()
    t.G8 = ctypes.cast(buf, ctypes.POINTER(ctypes.c_int))
    lib.init_g8.argtypes = [ctypes.POINTER(K.QED_kernel_temps)]
    lib.init_g8(ctypes.byref(t))
    assert np.array_equal(np.frombuffer(buf, dtype=np.int32), oracle_g8())
    tr = lambda *i: lib.diractrace(len(i), (ctypes.c_int * max(len(i), 1))(*i))
    assert tr() == 1 and tr(0) == 0 and tr(1, 1) == 1 and tr(0, 1) == 0
    assert tr(0, 0, 1, 1) == 1 and tr(0, 1, 0, 1) == -1 and tr(0, 1, 1, 0) == 1


def test_library_analytic_functions(lib):
    fx = np.load(FIX)
    for name in ("amu_heavlept", "amu_lightlept", "vac_pol"):
        got = np.array([getattr(lib, name)(a) for a in fx["fn_args"]])
        ref = fx[name]
        assert np.all(np.abs(got - ref) <= 1e-14 * np.abs(ref)), name
    for xv, ref in zip(fx["bessk_x"], fx["bessk"]):
        out = (ctypes.c_double * 5)()
        lib.bessk(4, xv, out)
        assert np.all(np.abs(np.array(out[:]) - ref) <= 1e-14 * np.abs(ref)), xv
