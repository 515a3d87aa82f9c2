"""The table readers and writers of the C ABI (read_ff, read_TAYLORX,
read_TAYLORY, write_ff, write_TAYLORX, write_TAYLORY; the reference's
src/LIBFILES/io.c:42-412): a read-then-write round trip reproduces the
table files byte for byte, and a corrupted file is refused by its checksum.
Host code only: no kernel runs."""
import ctypes
import os
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PRECOMP = os.path.join(ROOT, "kqed_gb300", "PRECOMP")


@pytest.fixture(scope="module")
def lib():
    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300 as K
    L = K.lib()
    G = ctypes.POINTER(K.Grid_coeffs)
    for n in ("read_ff", "read_TAYLORX", "read_TAYLORY"):
        getattr(L, n).argtypes = [G]
        getattr(L, n).restype = ctypes.c_int
    for n in ("write_ff", "write_TAYLORX", "write_TAYLORY"):
        getattr(L, n).argtypes = [G]
        getattr(L, n).restype = None
    return L


def _read_all(L, libdir):
    import kqed_gb300 as K
    old = os.environ.get("KQED_LIB_PATH")
    os.environ["KQED_LIB_PATH"] = libdir
    try:
        g = K.Grid_coeffs()
        rc = (L.read_ff(ctypes.byref(g)), L.read_TAYLORX(ctypes.byref(g)),
              L.read_TAYLORY(ctypes.byref(g)))
    finally:
        if old is None:
            del os.environ["KQED_LIB_PATH"]
        else:
            os.environ["KQED_LIB_PATH"] = old
    return g, rc


def test_read_then_write_reproduces_the_files(lib, tmp_path, monkeypatch):
    g, rc = _read_all(lib, os.path.join(ROOT, "kqed_gb300"))
    assert rc == (0, 0, 0)
    assert (g.nstpx, g.NtayY, g.NY_tay, g.NtayX, g.NX_tay) == (g.nstpx, 23, 810, 14, 100)
    monkeypatch.chdir(tmp_path)
    os.mkdir("PRECOMP")
    lib.write_ff(ctypes.byref(g))
    lib.write_TAYLORX(ctypes.byref(g))
    lib.write_TAYLORY(ctypes.byref(g))
    for out, orig in (("FFxy_single_cksum2.bin", "FFxy_single_cksum.bin"),
                      ("taylorx_cksum.bin", "taylorx_cksum.bin"),
                      ("taylory_cksum.bin", "taylory_cksum.bin")):
        a = open(os.path.join("PRECOMP", out), "rb").read()
        b = open(os.path.join(PRECOMP, orig), "rb").read()
        assert a == b, out


def test_corrupted_table_is_refused(lib, tmp_path):
    d = tmp_path / "PRECOMP"
    d.mkdir()
    for n in ("FFxy_single_cksum.bin", "taylorx_cksum.bin", "taylory_cksum.bin"):
        shutil.copy(os.path.join(PRECOMP, n), d / n)
    for n in ("FFxy_single_cksum.bin", "taylorx_cksum.bin", "taylory_cksum.bin"):
        raw = bytearray(open(d / n, "rb").read())
        raw[len(raw) // 2] ^= 0x10
        open(d / n, "wb").write(bytes(raw))
    _, rc = _read_all(lib, str(tmp_path))
    assert rc == (1, 1, 1)
