"""The FP64 work model behind bench.py's roofline (`benchmarks/flops.py`):
its per-branch accounting of a lattice launch agrees with the oracle's own
classification of every (x, y) pair -- x = 0 / y = 0 / x = y pairs at the
axis cost, generic pairs (on or below the x grid, swapped or not) at
PER_K * Ktop + FIXED, zero kernels (x = y = 0) free, and for L2 / L3 the
x = 0 rows free (their terms cancel identically and the kernels skip
them).  The grid is given
the table's x extents and a constant Chebyshev length, so Ktop is the same
in every cell."""
import ctypes

import numpy as np

from _helpers import oracle, oracle_branch


def test_lattice_work_model_matches_oracle_branches():
    from benchmarks import flops as F
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    O = oracle()
    nstpx, nstpy = ctypes.c_int(), ctypes.c_int()
    lim = [ctypes.c_double() for _ in range(4)]
    assert O.oracle_grid(ctypes.byref(nstpx), ctypes.byref(nstpy),
                         *[ctypes.byref(v) for v in lim]) == 0
    xlo, xhi = lim[0].value, lim[1].value
    XX = np.linspace(xlo, xhi, nstpx.value)
    nf = 20
    nfx = [nf] * nstpx.value
    ys = lattice_sites(6, 0.25)
    xs = np.vstack([diagonal_x(4, 0.25), [[0.3, -0.2, 0.5, 0.1]], [[0.25, 0.0, 0.0, -0.5]]])
    assert np.all(np.linalg.norm(xs, axis=1) <= xhi)
    T = F.table()
    per_gen = T["PER_K"] * (nf + 2) + T["FIXED"]
    for variant in (0, 2):
        expect = 0.0
        for xv in xs:
            if variant >= 2 and float(xv @ xv) < 1e-28:
                continue
            code = oracle_branch(np.repeat(xv[None, :], len(ys), 0), ys)
            base = code & 7
            assert not np.any(code & 16)
            expect += T["AXIS"] * np.isin(base, (1, 2, 3)).sum()
            expect += per_gen * np.isin(base, (4, 5)).sum()
            expect += len(ys) * (T["CONTRACT"] + (T["CONTRACT_EXTRA"] if variant else 0.0))
        got = F.lattice_flops(xs, ys, XX, nfx, variant)
        assert got == expect, (variant, got, expect)
