"""FP64 work model of the fused lattice kernel, per pair and branch.

The figures are the FP64 operations the kernel performs per (x, y) pair
(add/sub/mul = 1, fma = 2; divisions and square roots count as the FMA
sequences they compile to), measured once per kernel version with ncu's
executed-instruction counters on branch-uniform cases
(`python -m benchmarks.calibrate`, summary in profiles/) and frozen here.
A generic pair costs PER_K * Ktop + FIXED, Ktop = max(nfx[ix], nfx[ix+1]) + 2
being the number of Chebyshev steps of its x cell; an x=0 / y=0 / x=y pair
costs AXIS.  CONTRACT is the per-pair contraction with Pi (and the per-site
and per-x terms of L1..L3).
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "flops_table.json")

# defaults: hand count of the kernel's FP64 operations (replaced by the
# calibrated table when present)
_DEFAULT = {"PER_K": 573.0, "FIXED": 9000.0, "AXIS": 6500.0, "CONTRACT": 768.0,
            "CONTRACT_EXTRA": 768.0, "source": "hand count"}


def table():
    if os.path.exists(TABLE):
        with open(TABLE) as f:
            return json.load(f)
    return dict(_DEFAULT)


def lattice_flops(xs, ys, XX, nfx, variant, model=None):
    """Flops of one fused lattice launch over all (x_k, y_n): the FP64-
    equivalent model (model None), or one kernel's executed operations on one
    pipe, model = "record_fp64", "record_fp32", "assembly_fp64",
    "assembly_fp32" (calibrated per kernel and pipe)."""
    T = table()
    if model is not None:
        K = T.get("kernels", {}).get(model)
        if K is None:
            return None
        T = dict(K, CONTRACT=0.0, CONTRACT_EXTRA=0.0)
    xs = np.asarray(xs)
    ys = np.asarray(ys)
    nx, ny = len(xs), len(ys)
    ynz = (ys * ys).sum(1) >= 1e-28
    total = 0.0
    for k in range(nx):
        xv = xs[k]
        xz = float(xv @ xv) < 1e-28
        same = ((ys - xv) ** 2).sum(1) < 1e-28
        if xz and variant >= 2:
            continue            # every L2 / L3 term at x = 0 cancels: the pairs are skipped
        if xz:
            n_axis = int(ynz.sum())
            n_gen = 0
        else:
            n_axis = int((~ynz).sum() + same.sum())
            n_gen = ny - n_axis
            X = np.sqrt(max(float(xv @ xv), 1e-7))
            ix = int(np.searchsorted(XX, X, side="right") - 1)
            ix = max(0, min(ix, len(XX) - 1))
            ix2 = min(ix + 1, len(XX) - 1)
            ktop = max(nfx[ix], nfx[ix2]) + 2
            if X > XX[-1]:
                n_gen = 0
            total += n_gen * (T["PER_K"] * ktop + T["FIXED"])
        total += n_axis * T["AXIS"]
        total += ny * (T["CONTRACT"] + (T["CONTRACT_EXTRA"] if variant else 0.0))
    return total
