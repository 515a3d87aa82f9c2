"""Generates the golden fixtures under tests/golden/ (run here, where the
reference sources exist; the fixtures travel, the reference does not).

1. reg_axis.npz -- the table-independent columns of the reference's own
   regression files (PRECOMP/REGexample2.txt, REGexample10.txt, printed with
   %lg): kernels with one argument zero, which use only the Taylor tables and
   the x grid.  Inputs follow src/amu_forlattice.c:119-156 (example2) and
   :358-379 (example10).
2. ref_synth.npz -- outputs of the reference library itself (compiled from its
   own sources by oracle/Makefile, scalar flavour) on the synthetic
   form-factor table, for seeded pairs covering every branch, plus the table's
   checksums so a test can confirm the same table is in use.

3. ref_composite.npz -- the reference's composite kernels on seeded pairs.
4. ref_pihat.npz -- the reference's perturbative lepton-loop Pi-hat.

Usage: python tests/golden/make_golden.py [axis] [synth] [composite] [pihat]
       (default: all three; needs `make -C oracle ref`)
"""
import ctypes
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
from _helpers import reference_root  # noqa: E402

REF = reference_root()
if REF is None:
    sys.exit("make_golden.py: set KQED_REFERENCE to the reference checkout")


def parse_reg(path):
    """Rows 'rhosig= r mu= m nu= n lda= l v1 v2' -> array [nblocks, 384, 2]."""
    vals = []
    for ln in open(path):
        if ln.startswith("rhosig"):
            p = ln.split()
            vals.append((float(p[8]), float(p[9])))
    v = np.array(vals)
    return v.reshape(-1, 384, 2)


def reg_axis():
    ex2 = parse_reg(os.path.join(REF, "PRECOMP", "REGexample2.txt"))
    ex10 = parse_reg(os.path.join(REF, "PRECOMP", "REGexample10.txt"))
    vi = (1.228, 0.209243, 0.0484223)
    co, si = np.cos(vi[1]), np.sin(vi[1])
    yv = np.array([0, 0, 0, vi[2]])
    xv = np.array([0, 0, vi[0] * si, vi[0] * co])
    x10 = np.array([0.1, 0.1, 0.1, 0.1])
    z = np.zeros(4)
    # (x, y, golden L0(x,y)) for the four table-independent columns
    cases_x = np.array([z, z, x10, xv])
    cases_y = np.array([yv, x10, z, z])
    golden = np.array([ex2[0, :, 1], ex10[0, :, 0], ex10[0, :, 1], ex2[1, :, 1]])
    np.savez(os.path.join(HERE, "reg_axis.npz"), x=cases_x, y=cases_y, L0=golden)


def seeded_pairs():
    """Seeded pairs that cover every branch of L0."""
    rng = np.random.default_rng(20240601)
    gen_x = rng.uniform(-2, 2, (96, 4))
    gen_y = rng.uniform(-2, 2, (96, 4))
    d = rng.uniform(-1, 1, (32, 4))
    s = 10 ** rng.uniform(-6, -3, 32)
    small = d * s[:, None]
    other = rng.uniform(-2, 2, (32, 4))
    xs = [gen_x, small[:16], other[16:]]
    ys = [gen_y, other[:16], small[16:]]
    # exact special cases: x=0, y=0, x=y, both zero, far outside the grid
    big = np.array([[4.0, 4.0, 4.0, 4.0]])
    sp_x = np.vstack([np.zeros((1, 4)), gen_x[:2], gen_x[2:4], np.zeros((1, 4)), big, gen_x[4:5]])
    sp_y = np.vstack([gen_y[:1], np.zeros((2, 4)), gen_x[2:4], np.zeros((1, 4)), gen_y[5:6], big])
    xs.append(sp_x)
    ys.append(sp_y)
    # the reference's own example inputs (src/amu_forlattice.c:209-314)
    fac = 0.046241301098278
    ex_x = np.array([[1, 1, 1, 1.1], [0.001] * 4, [1 * fac, 3 * fac, 3 * fac, 52 * fac],
                     [0.001] * 4])
    ex_y = np.array([[1, 1, 1, 1], [1, 1, 1, 1], [fac] * 4, [0.001, 0.001, 0.001, -0.001]])
    xs += [ex_x, ex_y]
    ys += [ex_y, ex_x]
    return np.vstack(xs), np.vstack(ys)


def table_checksums(path):
    with open(path, "rb") as f:
        f.seek(-16, os.SEEK_END)
        return np.array(struct.unpack("<4I", f.read(16)), dtype=np.uint32)


def ref_synth():
    os.environ["KQEDREF_PATH"] = os.path.join(ROOT, "kqed_gb300")
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libkqedref_scalar.so"))
    assert lib.ref_init() == 0, "reference initialise() failed"
    dp = ctypes.POINTER(ctypes.c_double)
    x, y = seeded_pairs()
    out = {}
    for v in range(4):
        o = np.zeros((len(x), 384))
        lib.ref_kernel(v, len(x), x.ctypes.data_as(dp), y.ctypes.data_as(dp),
                       o.ctypes.data_as(dp), 1)
        out["L%d" % v] = o
    ck = table_checksums(os.path.join(ROOT, "kqed_gb300", "PRECOMP", "FFxy_single_cksum.bin"))
    np.savez_compressed(os.path.join(HERE, "ref_synth.npz"), x=x, y=y, table_cksum=ck, **out)


def ref_composite():
    """3. ref_composite.npz -- the reference's composite kernels
    (src/LIBFILES/all_kernels.c, con_kernel.c, sub_kernel.c, SYMXY.c,
    SYMXY0.c, kernels.c:181-231) through the same library, two of the
    composite_pairs() per composite, with each pair's term scale (the largest
    |L0| the composite combines, from the reference's own L0)."""
    from _helpers import (COMPOSITE_SIZE, composite_masses, composite_pairs,  # noqa: E402
                          composite_scale)
    os.environ["KQEDREF_PATH"] = os.path.join(ROOT, "kqed_gb300")
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libkqedref_scalar.so"))
    assert lib.ref_init() == 0, "reference initialise() failed"
    dp = ctypes.POINTER(ctypes.c_double)

    def ref_l0(a, b):
        a = np.ascontiguousarray(a)
        b = np.ascontiguousarray(b)
        o = np.zeros((len(a), 384))
        lib.ref_kernel(0, len(a), a.ctypes.data_as(dp), b.ctypes.data_as(dp),
                       o.ctypes.data_as(dp), 1)
        return o

    px, py = composite_pairs()
    out = {}
    for w in range(len(COMPOSITE_SIZE)):
        sel = [w % len(px), (w + 3) % len(px)]
        x, y = np.ascontiguousarray(px[sel]), np.ascontiguousarray(py[sel])
        M = composite_masses(w)
        o = np.zeros((2, COMPOSITE_SIZE[w]))
        assert lib.ref_composite(w, M.ctypes.data_as(dp), 2, x.ctypes.data_as(dp),
                                 y.ctypes.data_as(dp), o.ctypes.data_as(dp), 1) == 0
        out["x%d" % w], out["y%d" % w], out["out%d" % w] = x, y, o
        out["scale%d" % w] = composite_scale(w, x, y, ref_l0)
    np.savez_compressed(os.path.join(HERE, "ref_composite.npz"), **out)


def pihat_pairs():
    """seeded pairs for the perturbative Pi-hat: generic, short and long
    separations, and the reference's lepton-loop check points
    (src/amu_forlattice.c:80-96, scaled by the mass ratio 2)"""
    rng = np.random.default_rng(8080)
    x = rng.uniform(-1.5, 1.5, (6, 4))
    y = rng.uniform(-1.5, 1.5, (6, 4))
    x[1] = 0.02 * x[1]
    y[2] = x[2] + 0.01 * y[2]
    pts = []
    for xm, b, ym in ((0.405, 0.005 + np.pi / 4, 0.205), (0.805, 0.005 + np.pi / 2, 0.605)):
        pts.append((2 * np.array([0, 0, xm * np.sin(b), xm * np.cos(b)]), 2 * np.array([0, 0, 0, ym])))
    x = np.vstack([x] + [p[0][None] for p in pts])
    y = np.vstack([y] + [p[1][None] for p in pts])
    return x, y


def ref_pihat():
    """4. ref_pihat.npz -- the reference's perturbative lepton-loop Pi-hat
    (ipihatFermLoop_antisym and pihat1, src/LIBFILES/pi_pert.c) and its
    analytic functions, through the same library"""
    os.environ["KQEDREF_PATH"] = os.path.join(ROOT, "kqed_gb300")
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libkqedref_scalar.so"))
    assert lib.ref_init() == 0, "reference initialise() failed"
    dp = ctypes.POINTER(ctypes.c_double)
    x, y = pihat_pairs()
    anti = np.zeros((len(x), 384))
    assert lib.ref_pihat(len(x), x.ctypes.data_as(dp), y.ctypes.data_as(dp),
                         anti.ctypes.data_as(dp), 1) == 0
    raw = np.zeros((2, 1280))
    for i in range(2):
        xi, yi = np.ascontiguousarray(x[i]), np.ascontiguousarray(y[i])
        assert lib.ref_pihat1(xi.ctypes.data_as(dp), yi.ctypes.data_as(dp),
                              raw[i].ctypes.data_as(dp)) == 0
    for f in ("amu_heavlept", "amu_lightlept", "vac_pol"):
        getattr(lib, f).restype = ctypes.c_double
        getattr(lib, f).argtypes = [ctypes.c_double]
    args = np.array([0.5, 2.0, 1.0 / 206.768262, 16.8])
    heav = np.array([lib.amu_heavlept(a) for a in args])
    light = np.array([lib.amu_lightlept(a) for a in args])
    vac = np.array([lib.vac_pol(a) for a in args])
    bess = np.zeros((5, 6))
    lib.bessk.argtypes = [ctypes.c_int, ctypes.c_double, dp]
    bx = np.array([0.05, 0.7, 2.0, 2.5, 9.0])
    for i, v in enumerate(bx):
        lib.bessk(4, v, bess[i].ctypes.data_as(dp))
    np.savez_compressed(os.path.join(HERE, "ref_pihat.npz"), x=x, y=y, pihat=anti, pihat1=raw,
                        fn_args=args, amu_heavlept=heav, amu_lightlept=light, vac_pol=vac,
                        bessk_x=bx, bessk=bess[:, :5])


if __name__ == "__main__":
    if not os.path.isdir(REF):
        sys.exit("reference sources not found at %s" % REF)
    parts = sys.argv[1:] or ["axis", "synth", "composite", "pihat"]
    if "axis" in parts:
        reg_axis()
    if "synth" in parts:
        ref_synth()
    if "composite" in parts:
        ref_composite()
    if "pihat" in parts:
        ref_pihat()
    print("wrote", os.listdir(HERE))
