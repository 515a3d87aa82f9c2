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
