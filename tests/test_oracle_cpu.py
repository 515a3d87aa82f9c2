"""The oracle, pinned against the reference's own golden vectors, the
reference library's outputs on the synthetic table, and the reference's
identity tests (src/amu_forlattice.c examples 3, 9, 11, 15).  CPU only."""
import os
import shutil
import struct

import numpy as np
import pytest

from _helpers import (GOLDEN, PKG, REF_SO, norm_rel, oracle, oracle_branch, oracle_kernel)


def _taylor_cksums(path):
    """recompute the rank-rotated CRC32C pair of a Taylor file with a
    byte-wise CRC (independent of the C implementations)"""
    poly = 0x82F63B78
    tab = []
    for i in range(256):
        c = i
        for _ in range(8):
            c = (c >> 1) ^ poly if c & 1 else c >> 1
        tab.append(c)
    b = open(path, "rb").read()
    n = struct.unpack_from("<i", b, 4)[0]
    off = 8
    a = bb = 0
    for r in range(n):
        m = struct.unpack_from("<i", b, off)[0]
        off += 4
        w = 0
        for byte in b[off:off + 8 * m]:
            w = tab[(w ^ byte) & 0xFF] ^ (w >> 8)
        off += 8 * m
        r29, r31 = r % 29, r % 31
        a ^= ((w << r29) | (w >> (32 - r29))) & 0xFFFFFFFF if r29 else w
        bb ^= ((w << r31) | (w >> (32 - r31))) & 0xFFFFFFFF if r31 else w
    return (a, bb), struct.unpack_from("<II", b, off)


@pytest.mark.parametrize("name", ["taylorx_cksum.bin", "taylory_cksum.bin"])
def test_taylor_table_checksum_kat(name):
    computed, stored = _taylor_cksums(os.path.join(PKG, "PRECOMP", name))
    assert computed == stored


def test_synthetic_table_is_the_fixture_table():
    oracle()
    from kqed_gb300 import build as B
    with open(os.path.join(PKG, "PRECOMP", "FFxy_single_cksum.bin"), "rb") as f:
        f.seek(-16, os.SEEK_END)
        tail = struct.unpack("<4I", f.read(16))
    fx = np.load(os.path.join(GOLDEN, "ref_synth.npz"))
    assert tuple(int(v) for v in fx["table_cksum"]) == tail
    assert "%08x %08x %08x %08x" % tail == B.SYNTH_CKSUM


def test_oracle_matches_reference_outputs_on_synthetic_table():
    """fixtures made by the reference library itself (tests/golden/make_golden.py)"""
    fx = np.load(os.path.join(GOLDEN, "ref_synth.npz"))
    x, y = fx["x"], fx["y"]
    for v in range(4):
        ref = fx["L%d" % v]
        got = oracle_kernel(v, x, y, nthreads=1)
        zero_ref = np.abs(ref).max(1) == 0
        assert np.array_equal(zero_ref, np.abs(got).max(1) == 0), "zero-kernel pattern differs"
        err = norm_rel(got[~zero_ref], ref[~zero_ref])
        assert err.max() <= 1e-13, (v, err.max())


def test_oracle_matches_reference_golden_files():
    """PRECOMP/REGexample2.txt and REGexample10.txt columns that use only the
    Taylor tables and the x grid (printed with 6 significant digits)"""
    fx = np.load(os.path.join(GOLDEN, "reg_axis.npz"))
    got = oracle_kernel(0, fx["x"], fx["y"], nthreads=1)
    ref = fx["L0"]
    for g, r in zip(got, ref):
        scale = np.abs(r).max()
        assert np.all(np.abs(g - r) <= 5e-6 * np.abs(r) + 1e-6 * scale)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")
def test_oracle_matches_live_reference():
    import ctypes
    os.environ["KQEDREF_PATH"] = PKG
    L = ctypes.CDLL(REF_SO)
    assert L.ref_init() == 0
    dp = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(7)
    x = rng.uniform(-3, 3, (512, 4))
    y = rng.uniform(-3, 3, (512, 4))
    for v in range(4):
        ref = np.zeros((512, 384))
        L.ref_kernel(v, 512, x.ctypes.data_as(dp), y.ctypes.data_as(dp), ref.ctypes.data_as(dp), 0)
        got = oracle_kernel(v, x, y)
        nz = np.abs(ref).max(1) > 0
        assert np.array_equal(nz, np.abs(got).max(1) > 0)
        assert norm_rel(got[nz], ref[nz]).max() <= 1e-13


def _mulam(k):
    return np.swapaxes(k.reshape(-1, 6, 4, 4, 4), 2, 4).reshape(-1, 384)


def test_identity_ex3_vanishing_kernels():
    """L0(0,0)=0, L1(x,x)=0, L2(0,y)=L2(x,0)=0, L3(x,x)=L3(0,y)=L3(y,y)=L3(0,x)=0
    (src/amu_forlattice.c:158-206)"""
    z = np.zeros((1, 4))
    x = np.array([[1.0, 2.0, 3.0, 4.0]]) * 0.3
    y = np.array([[4.0, 3.0, 2.0, 1.0]]) * 0.3
    cases = [(0, z, z), (1, x, x), (2, z, y), (2, x, z), (3, x, x), (3, z, y), (3, z, x), (3, y, y)]
    for v, a, b in cases:
        assert np.abs(oracle_kernel(v, a, b)).max() <= 1e-14


def test_identity_ex9_diagonal_is_swapped_axis():
    """L(x,x) = -L_{mu<->lambda}(x,0) (src/amu_forlattice.c:317-355)"""
    th = np.arange(0.1, 1.0, 0.05)
    x = np.outer(th, [1, 2, 3, 4])
    kxx = oracle_kernel(0, x, x)
    kx0 = oracle_kernel(0, x, np.zeros_like(x))
    assert np.abs(kxx + _mulam(kx0)).max() <= 1e-14


def test_identity_ex11_parity():
    """L^i(x,y) = -L^i(-x,-y) on the reference's 2x2x2x4 pretend lattice
    (src/amu_forlattice.c:382-457)"""
    idx = np.arange(32)
    c = np.stack([idx % 2, (idx // 2) % 2, (idx // 4) % 2, idx // 8], 1).astype(float)
    c[:, 3] = np.where(c[:, 3] > 2, c[:, 3] - 4, c[:, 3])
    X = np.repeat(c, 32, 0)
    Y = np.tile(c, (32, 1))
    for v in range(4):
        a = oracle_kernel(v, X, Y)
        b = oracle_kernel(v, -X, -Y)
        assert np.abs(a + b).max() <= 1e-14 * max(1.0, np.abs(a).max())


def test_identity_ex15_translation():
    """L(x-y,0) = -L(y-x,0) (src/amu_forlattice.c:692-742)"""
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (64, 4))
    y = rng.uniform(-1, 1, (64, 4))
    z = np.zeros_like(x)
    a = oracle_kernel(0, x - y, z)
    b = oracle_kernel(0, y - x, z)
    assert np.abs(a + b).max() <= 1e-14 * np.abs(a).max()


def test_branch_coverage_of_config1():
    from kqed_gb300.workloads import config1_pairs
    x, y = config1_pairs()
    code = oracle_branch(x, y)
    kinds = set(int(c) & 7 for c in code)
    assert 4 in kinds and 5 in kinds, kinds  # generic and Taylor-in-x
    assert np.any(code & 8)  # x <-> (x-y) swap


def test_corrupt_table_is_rejected(tmp_path):
    """a flipped byte must fail the checksum (src/LIBFILES/io.c:160-173)"""
    import ctypes
    oracle()
    d = tmp_path / "PRECOMP"
    d.mkdir()
    for n in ["taylorx_cksum.bin", "taylory_cksum.bin"]:
        shutil.copy(os.path.join(PKG, "PRECOMP", n), d / n)
    src = os.path.join(PKG, "PRECOMP", "FFxy_single_cksum.bin")
    b = bytearray(open(src, "rb").read())
    b[len(b) // 2] ^= 0x40
    (d / "FFxy_single_cksum.bin").write_bytes(bytes(b))
    O = ctypes.CDLL(os.path.join(os.path.dirname(PKG), "oracle", "_build", "liboracle.so"))
    O.oracle_load.argtypes = [ctypes.c_char_p]
    try:
        assert O.oracle_load(str(tmp_path).encode()) != 0
    finally:
        assert O.oracle_load(PKG.encode()) == 0


def test_synthetic_pi_generator_statistics():
    """The generated-Pi benchmark input: g values standardised (mean 0,
    variance 1 - 2^-16), bounded by 510 sqrt(3)/256, envelope 1 at x = y = 0,
    and distinct for distinct seeds, streams and x indices"""
    from _helpers import oracle_pi_synth
    x = np.zeros((1, 4))
    y = np.zeros((64, 4))
    g = oracle_pi_synth(x, y, seed=12345).ravel()
    assert abs(g.mean()) < 0.02 and abs(g.var() - 1.0) < 0.03
    assert np.abs(g).max() <= 510 * np.sqrt(3) / 256 + 1e-12
    q = np.round(g / (np.sqrt(3) / 256)).astype(int)
    assert np.allclose(q * (np.sqrt(3) / 256), g, rtol=0, atol=1e-13)
    assert not np.array_equal(g, oracle_pi_synth(x, y, seed=12346).ravel())
    assert not np.array_equal(g, oracle_pi_synth(x, y, seed=12345, stream=1).ravel())
    assert not np.array_equal(g, oracle_pi_synth(x, y, seed=12345, k0=1).ravel())
    y2 = np.array([[0.3, 0.0, 0.4, 0.0]])
    x2 = np.array([[0.0, 0.0, 0.0, 0.0]])
    p = oracle_pi_synth(x2, y2, seed=7)[0, 0]
    p0 = oracle_pi_synth(x, y2, seed=7)[0, 0]
    assert np.array_equal(p, p0)
    np.testing.assert_allclose(p / oracle_pi_synth(x, y2 * 0, seed=7)[0, 0], np.exp(-0.5), rtol=1e-15)


def _edge_pairs(xlo, xhi, ylo, yhi):
    """pairs on the branch and grid edges: y = c x (cb = +-1 exactly), x = -y,
    |x| or |y| on the first / last grid node, cb one ulp-scale away from +-1,
    tiny arguments, x = y + tiny, and lattice-diagonal pairs"""
    rng = np.random.default_rng(11)
    u = rng.normal(size=(16, 4))
    u /= np.linalg.norm(u, axis=1)[:, None]
    X, Y = [], []
    for i, c in enumerate((0.5, 2.0, -0.5, -2.0, -1.0)):
        X.append(u[i]); Y.append(c * u[i])
    for i, (rx, ry) in enumerate(((xlo, 1.0), (xhi, 1.0), (1.0, ylo), (1.0, yhi), (xlo, ylo))):
        X.append(rx * u[5 + i]); Y.append(ry * u[10 + i])
    w = np.array([1.0, 0.0, 0.0, 0.0]); p = np.array([0.0, 1.0, 0.0, 0.0])
    for eps in (1e-6, 1e-9):
        X.append(1.3 * w); Y.append(0.7 * (w + eps * p))
        X.append(1.3 * w); Y.append(-0.7 * (w + eps * p))
    for s in (1e-8, 1e-5):
        X.append(s * u[0]); Y.append(u[1])
        X.append(u[2]); Y.append(s * u[3])
    for d in (1e-10, 1e-6):
        X.append(u[4]); Y.append(u[4] + d * u[5])
    diag = np.ones(4) * 0.1
    for k, m in ((1, 2), (3, 1), (2, -2), (5, 7), (4, -1)):
        X.append(k * diag); Y.append(m * diag)
    return np.array(X), np.array(Y)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")
def test_oracle_matches_live_reference_on_edge_pairs():
    import ctypes
    os.environ["KQEDREF_PATH"] = PKG
    L = ctypes.CDLL(REF_SO)
    assert L.ref_init() == 0
    dp = ctypes.POINTER(ctypes.c_double)
    O = oracle()
    nstpx, nstpy = ctypes.c_int(), ctypes.c_int()
    lim = [ctypes.c_double() for _ in range(4)]
    assert O.oracle_grid(ctypes.byref(nstpx), ctypes.byref(nstpy),
                         *[ctypes.byref(v) for v in lim]) == 0
    x, y = _edge_pairs(*(v.value for v in lim))
    n = len(x)
    for v in range(4):
        ref = np.zeros((n, 384))
        L.ref_kernel(v, n, x.ctypes.data_as(dp), y.ctypes.data_as(dp), ref.ctypes.data_as(dp), 0)
        got = oracle_kernel(v, x, y)
        nz = np.abs(ref).max(1) > 0
        assert np.array_equal(nz, np.abs(got).max(1) > 0), v
        err = norm_rel(got[nz], ref[nz])
        assert err.max() <= 1e-13, (v, err.max(), int(np.argmax(err)))


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built here")
def test_oracle_follows_the_reference_portable_path_on_near_equal_pairs():
    """|x - y| = d |x|, d = 1e-10 .. 1e-2: the swap branch's rounding
    sensitivity grows like (|x| / |x - y|)^2 (the reference's own AVX2/FMA
    and portable builds differ by up to ~5e-2 here), yet the oracle, which
    restates the portable path's operation order without contraction, stays
    within 1e-14 of it"""
    import ctypes
    os.environ["KQEDREF_PATH"] = PKG
    L = ctypes.CDLL(REF_SO)
    assert L.ref_init() == 0
    dp = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(5)
    n = 64
    u = rng.uniform(-2, 2, (n, 4))
    w = rng.normal(size=(n, 4))
    w /= np.linalg.norm(w, axis=1)[:, None]
    for d in (1e-10, 1e-8, 1e-6, 1e-4, 1e-2):
        y = u + d * np.linalg.norm(u, axis=1)[:, None] * w
        ref = np.zeros((n, 384))
        L.ref_kernel(0, n, u.ctypes.data_as(dp), y.ctypes.data_as(dp), ref.ctypes.data_as(dp), 0)
        got = oracle_kernel(0, u, y)
        nz = np.abs(ref).max(1) > 0
        assert nz.all()
        assert norm_rel(got, ref).max() <= 1e-14, d
