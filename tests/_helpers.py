"""Shared test helpers: the oracle (CPU checker) and seeded inputs."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "kqed_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libkqedref_scalar.so")


def reference_root():
    """The reference checkout: the environment variable KQED_REFERENCE, else
    the one the build recorded in oracle/_ref/REFERENCE; None when neither
    names an existing directory (the tests that read it then skip)."""
    cand = os.environ.get("KQED_REFERENCE")
    if not cand:
        rec = os.path.join(ROOT, "oracle", "_ref", "REFERENCE")
        if os.path.exists(rec):
            cand = open(rec).read().strip()
    return cand if cand and os.path.isdir(os.path.join(cand, "src")) else None

_dp = ctypes.POINTER(ctypes.c_double)
_oracle = None


def ensure_table():
    from kqed_gb300 import build as B
    os.makedirs(B.OUT, exist_ok=True)
    B.ensure_table(B.build_synth())


def oracle():
    """The CPU oracle, loaded on the package's tables (built on first use)."""
    global _oracle
    if _oracle is None:
        ensure_table()
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True,
                       capture_output=True)
        O = ctypes.CDLL(ORACLE_SO)
        O.oracle_load.argtypes = [ctypes.c_char_p]
        if O.oracle_load(PKG.encode()) != 0:
            raise RuntimeError("oracle could not load the tables")
        _oracle = O
    return _oracle


def oracle_kernel(variant, x, y, nthreads=0):
    O = oracle()
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros((len(x), 384))
    assert O.oracle_kernel(variant, len(x), x.ctypes.data_as(_dp), y.ctypes.data_as(_dp),
                           out.ctypes.data_as(_dp), nthreads) == 0
    return out


def oracle_contract(variant, x, y, pi, nthreads=0):
    O = oracle()
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    pi = np.ascontiguousarray(pi, np.float64)
    dots = np.zeros(len(x))
    assert O.oracle_contract(variant, len(x), x.ctypes.data_as(_dp), y.ctypes.data_as(_dp),
                             pi.ctypes.data_as(_dp), dots.ctypes.data_as(_dp), nthreads) == 0
    return dots


def oracle_branch(x, y):
    O = oracle()
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    code = np.zeros(len(x), dtype=np.int32)
    O.oracle_branch(len(x), x.ctypes.data_as(_dp), y.ctypes.data_as(_dp),
                    code.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return code


def norm_rel(a, b, tau=1e-300):
    """Per-pair max_i |a_i - b_i| / max(|b|_inf, tau)."""
    a = np.asarray(a).reshape(len(b), -1)
    b = np.asarray(b).reshape(len(b), -1)
    return np.abs(a - b).max(1) / np.maximum(np.abs(b).max(1), tau)


def neumaier(v):
    s = 0.0
    c = 0.0
    for x in v:
        t = s + x
        c += (s - t) + x if abs(s) >= abs(x) else (x - t) + s
        s = t
    return s + c


def oracle_pi_synth(x, y, seed, stream=0, k0=0, n0=0):
    """The synthetic Pi of kqed_lattice_sum_synth, [nx][ny][384], from the
    oracle's restatement of the generator."""
    O = oracle()
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros((len(x), len(y), 384))
    O.oracle_pi_synth.argtypes = [ctypes.c_long, _dp, ctypes.c_long, _dp, ctypes.c_uint64,
                                  ctypes.c_uint32, ctypes.c_long, ctypes.c_long, _dp]
    assert O.oracle_pi_synth(len(x), x.ctypes.data_as(_dp), len(y), y.ctypes.data_as(_dp), seed,
                             stream, k0, n0, out.ctypes.data_as(_dp)) == 0
    return out


# the reference's composite kernels, numbered as enum kqed_composite
COMPOSITES = ["all_kernels", "all_Mkernels", "all_Mkernels_v2", "con_kernels",
              "con_kernels_v2", "con_kernelsM_L2", "sub_kernelsM_L2", "SYMXY", "SYMXY_v2",
              "SYMXY0", "SYMXY0_v2", "Mkernel_L2"]
COMPOSITE_SIZE = [3072, 3072, 3072, 3072, 4608, 4608, 4608, 3072, 1536, 3072, 1536, 384]


def oracle_composite(which, x, y, M=None, nthreads=0):
    """out[n][size]: the oracle's restatement of composite `which`."""
    O = oracle()
    O.oracle_composite.argtypes = [ctypes.c_int, _dp, ctypes.c_long, _dp, _dp, _dp, ctypes.c_int]
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    Mv = np.ascontiguousarray(np.zeros(4) if M is None else np.atleast_1d(M), np.float64)
    out = np.zeros((len(x), COMPOSITE_SIZE[which]))
    assert O.oracle_composite(which, Mv.ctypes.data_as(_dp), len(x), x.ctypes.data_as(_dp),
                              y.ctypes.data_as(_dp), out.ctypes.data_as(_dp), nthreads) == 0
    return out


# the L0 evaluations each composite combines (reference function bodies),
# as (first argument, second argument) over x, y, 0, x-y, y-x, -y
_ALLS = [("x", "y"), ("y", "x"), ("x", "0"), ("0", "x"), ("y", "0"), ("0", "y")]
_CONS = [("x", "y"), ("y", "x"), ("x", "x-y"), ("x", "0"), ("0", "x"), ("y", "0"), ("0", "y"),
         ("x-y", "0"), ("0", "x-y")]
_CONMS = [("x", "y"), ("y", "x"), ("x", "x-y"), ("x", "0"), ("0", "x"), ("y", "0"), ("0", "y"),
          ("0", "x-y")]
_SYM0S = [("x", "y"), ("y", "x"), ("x-y", "x"), ("y-x", "y"), ("x", "x-y"), ("y", "y-x"),
          ("x", "0"), ("0", "x"), ("y", "0"), ("0", "y"), ("x-y", "0"), ("0", "x-y")]
COMPOSITE_SOURCES = [_ALLS, _ALLS, _ALLS + [("x", "-y")], _CONS, _CONS, _CONMS, _CONMS, _ALLS,
                     _ALLS, _SYM0S, _SYM0S, [("x", "y"), ("0", "y"), ("x", "0")]]


def derived_arg(code, x, y):
    return {"x": x, "y": y, "0": np.zeros_like(x), "x-y": x - y, "y-x": -(x - y), "-y": -y}[code]


def composite_scale(which, x, y, l0=None):
    """Per pair, the largest |L0| among the evaluations composite `which`
    combines: the floating-point scale of its linear combinations (an output
    can be far smaller than its terms, e.g. when |x| is tiny).  l0(a, b) ->
    [n][384], the oracle's by default."""
    l0 = l0 or (lambda a, b: oracle_kernel(0, a, b))
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    s = np.zeros(len(x))
    for a, b in COMPOSITE_SOURCES[which]:
        s = np.maximum(s, np.abs(l0(derived_arg(a, x, y), derived_arg(b, x, y))).max(1))
    return s


# the masses of the reference's own calls (src/amu_forlattice.c:1411, 1094)
COMPOSITE_M4 = np.array([0.0, 0.5, 1.0, 1.5])
COMPOSITE_M1 = np.array([0.7])


def composite_masses(which):
    return COMPOSITE_M1 if which == 11 else COMPOSITE_M4


def composite_pairs():
    """Seeded pairs covering the branches the composites reach: generic,
    the x <-> (x-y) swap, |x| below the first grid node, x = 0, y = 0,
    x = y, y on the ray of x, and the reference's stress-test point."""
    rng = np.random.default_rng(424242)
    g = rng.uniform(-1.5, 1.5, (2, 4))
    x = np.array([g[0], [0.9, 0.5, -0.4, 0.7], 2e-4 * g[1], np.zeros(4), [0.3, -1.2, 0.8, 0.1],
                  [1.1, 0.2, -0.6, 0.4], [0.5, 0.25, -0.5, 1.0], [1.0, 2.0, 3.0, 4.0]])
    y = np.array([g[1], [0.8, 0.45, -0.3, 0.75], [-0.9, 0.3, 1.0, 0.5], [0.6, -0.2, 0.4, 1.3],
                  np.zeros(4), [1.1, 0.2, -0.6, 0.4], [0.3, 0.15, -0.3, 0.6], [1.0, 1.0, 1.0, 1.0]])
    return x, y


def oracle_pihat(x, y, nthreads=0):
    """[n][384]: the oracle's ipihatFermLoop_antisym(x[i], y[i])"""
    O = oracle()
    O.oracle_pihat.argtypes = [ctypes.c_long, _dp, _dp, _dp, ctypes.c_int]
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros((len(x), 384))
    assert O.oracle_pihat(len(x), x.ctypes.data_as(_dp), y.ctypes.data_as(_dp),
                          out.ctypes.data_as(_dp), nthreads) == 0
    return out


def oracle_g8():
    O = oracle()
    out = np.zeros(65536, dtype=np.int32)
    O.oracle_g8(out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return out
