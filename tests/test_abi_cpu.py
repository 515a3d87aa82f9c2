"""The C-ABI library: it loads, exports every entry point include/kqed.h
declares, keeps the reference's struct layout, and reports load errors the
way the reference does (return 1, message).  CPU only: no kernel runs."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest
from _helpers import reference_root

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "kqed.h")
REF_ROOT = reference_root()
REF_HDR = os.path.join(REF_ROOT, "src", "HEADERS", "KQED.h") if REF_ROOT else ""


@pytest.fixture(scope="module")
def lib():
    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300
    return kqed_gb300.lib()


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", src,
                       flags=re.M)
    return sorted(set(names))


def test_header_declares_the_reference_api():
    names = declared_functions()
    for n in ["initialise", "free_QED_temps", "QED_kernel_L0", "QED_kernel_L1", "QED_kernel_L2",
              "QED_kernel_L3", "kqed_kernel_batch", "kqed_lattice_sum"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True,
                         text=True, check=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def _offsets_c(include_dir, header, tmpdir):
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "%s"
int main(void){
  printf("%%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu\n", sizeof(struct QED_kernel_temps),
    offsetof(struct QED_kernel_temps, G8), offsetof(struct Grid_coeffs, XX),
    offsetof(struct Grid_coeffs, nstpx), offsetof(struct Grid_coeffs, TX),
    offsetof(struct Grid_coeffs, TY), offsetof(struct Grid_coeffs, PC),
    offsetof(struct Grid_coeffs, nfx));
  return 0; }
''' % header
    c = os.path.join(tmpdir, "off.c")
    open(c, "w").write(prog)
    exe = os.path.join(tmpdir, "off")
    subprocess.run(["gcc", "-I", include_dir, "-o", exe, c], check=True, capture_output=True)
    return subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()


def test_struct_layout_matches_ctypes(tmp_path):
    import kqed_gb300 as K
    got = _offsets_c(os.path.dirname(HDR), "kqed.h", str(tmp_path))
    T, G = K.QED_kernel_temps, K.Grid_coeffs
    want = [ctypes.sizeof(T), T.G8.offset, G.XX.offset, G.nstpx.offset, G.TX.offset,
            G.TY.offset, G.PC.offset, G.nfx.offset]
    assert [int(v) for v in got] == want


@pytest.mark.skipif(not REF_HDR or not os.path.exists(REF_HDR),
                    reason="reference headers not present (KQED_REFERENCE unset)")
def test_struct_layout_matches_reference(tmp_path):
    """sizeof/offsets of struct QED_kernel_temps equal the reference's
    (src/HEADERS/KQED.h:69-93), so it can be passed by value unchanged"""
    inc = tmp_path / "inc"
    inc.mkdir()
    shutil.copy(os.path.join(ROOT, "oracle", "ref", "config.h"), inc / "config.h")
    prog_inc = "-I" + os.path.dirname(REF_HDR)
    ours = _offsets_c(os.path.dirname(HDR), "kqed.h", str(tmp_path))
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "KQED.h"
int main(void){
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(struct QED_kernel_temps),
    offsetof(struct QED_kernel_temps, G8), offsetof(struct Grid_coeffs, XX),
    offsetof(struct Grid_coeffs, nstpx), offsetof(struct Grid_coeffs, TX),
    offsetof(struct Grid_coeffs, TY), offsetof(struct Grid_coeffs, PC),
    offsetof(struct Grid_coeffs, nfx));
  return 0; }
'''
    (tmp_path / "r.c").write_text(src)
    subprocess.run(["gcc", "-I", str(inc), prog_inc, "-o", str(tmp_path / "r"),
                    str(tmp_path / "r.c")], check=True, capture_output=True)
    ref = subprocess.run([str(tmp_path / "r")], capture_output=True, text=True,
                         check=True).stdout.split()
    assert ours == ref


def test_initialise_rejects_a_corrupt_table(lib, tmp_path):
    import kqed_gb300 as K
    pkg = os.path.dirname(K.__file__)
    d = tmp_path / "PRECOMP"
    d.mkdir()
    for n in ["taylorx_cksum.bin", "taylory_cksum.bin"]:
        shutil.copy(os.path.join(pkg, "PRECOMP", n), d / n)
    b = bytearray(open(os.path.join(pkg, "PRECOMP", "FFxy_single_cksum.bin"), "rb").read())
    b[-100] ^= 1
    (d / "FFxy_single_cksum.bin").write_bytes(bytes(b))
    old = os.environ.get("KQED_LIB_PATH")
    os.environ["KQED_LIB_PATH"] = str(tmp_path)
    try:
        t = K.QED_kernel_temps()
        assert lib.initialise(ctypes.byref(t)) == 1
        assert b"checksum" in lib.kqed_last_error()
        assert not t.Grid.PC
    finally:
        if old is None:
            del os.environ["KQED_LIB_PATH"]
        else:
            os.environ["KQED_LIB_PATH"] = old


def test_initialise_reports_missing_table(lib, tmp_path):
    import kqed_gb300 as K
    old = os.environ.get("KQED_LIB_PATH")
    os.environ["KQED_LIB_PATH"] = str(tmp_path)
    try:
        t = K.QED_kernel_temps()
        assert lib.initialise(ctypes.byref(t)) == 1
        assert b"Cannot find" in lib.kqed_last_error()
    finally:
        if old is None:
            del os.environ["KQED_LIB_PATH"]
        else:
            os.environ["KQED_LIB_PATH"] = old


def test_batch_rejects_uninitialised_tables(lib):
    import kqed_gb300 as K
    t = K.QED_kernel_temps()
    dp = ctypes.POINTER(ctypes.c_double)
    assert lib.kqed_kernel_batch(ctypes.byref(t), 0, 0, None, None, None, None, 0) == 1
    assert b"not initialised" in lib.kqed_last_error()


def test_pinned_contains_rejects_foreign_memory(lib):
    """the range query answers without a GPU: memory that kqed_pinned_alloc
    did not hand out is never taken for page-locked, device-mapped memory"""
    import numpy as np
    a = np.zeros(64)
    lib.kqed_pinned_contains.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    assert lib.kqed_pinned_contains(ctypes.c_void_p(a.ctypes.data), a.nbytes) == 0
    assert lib.kqed_pinned_contains(None, 8) == 0
    assert lib.kqed_pinned_contains(ctypes.c_void_p(a.ctypes.data), 0) == 0


def test_batch_structs_match_ctypes(tmp_path):
    """struct kqed_lattice_job / kqed_batch_info as the C compiler lays
    them out equal the ctypes mirrors the Python binding passes"""
    import kqed_gb300 as K
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "kqed.h"
int main(void){
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(struct kqed_lattice_job),
    offsetof(struct kqed_lattice_job, d_pi), offsetof(struct kqed_lattice_job, pi_stream),
    offsetof(struct kqed_lattice_job, d_sums), sizeof(struct kqed_batch_info),
    offsetof(struct kqed_batch_info, tuned_ms));
  return 0; }
'''
    c = tmp_path / "b.c"
    c.write_text(prog)
    exe = str(tmp_path / "b")
    subprocess.run(["gcc", "-I", os.path.dirname(HDR), "-o", exe, str(c)], check=True,
                   capture_output=True)
    got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True,
                                          check=True).stdout.split()]
    J, I = K.LatticeJob, K.BatchInfo
    assert got == [ctypes.sizeof(J), J.d_pi.offset, J.pi_stream.offset, J.d_sums.offset,
                   ctypes.sizeof(I), I.tuned_ms.offset]


def test_c_program_links_every_entry_point(lib, tmp_path):
    """a C caller (the reference's language) compiles against include/kqed.h,
    links libkqed_gb300.so and resolves every declared entry point; it then
    calls only kqed_last_error and kqed_launch_count (no GPU work)"""
    names = declared_functions()
    c = tmp_path / "link.c"
    c.write_text(
        "#include <stdio.h>\n#include \"kqed.h\"\n"
        "typedef void (*fp)(void);\n"
        "int main(void) {\n"
        "  fp f[] = {" + ", ".join("(fp)%s" % n for n in names) + "};\n"
        "  int n = 0;\n"
        "  for (unsigned i = 0; i < sizeof(f) / sizeof(f[0]); i++) n += f[i] != 0;\n"
        "  printf(\"%d %llu [%s]\\n\", n, (unsigned long long)kqed_launch_count(),"
        " kqed_last_error());\n"
        "  return 0;\n}\n")
    libdir = os.path.dirname(lib._name)
    exe = str(tmp_path / "link")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HDR), "-o",
                        exe, str(c), "-L" + libdir, "-lkqed_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == len(names) and int(out[1]) == 0


def test_out_argument_is_checked_before_any_call():
    """kernel_batch / composite_batch write into a caller's `out` only when it
    is a C-contiguous float64 array of the result's shape"""
    import numpy as np
    import kqed_gb300 as K
    x = np.zeros((3, 4))
    for bad in (np.zeros((3, 383)), np.zeros((3, 384), dtype=np.float32),
                np.zeros((384, 3)).T):
        with pytest.raises(ValueError):
            K.kernel_batch(None, 0, x, x, out=bad)
    with pytest.raises(ValueError):
        K.composite_batch(None, 0, x, x, out=np.zeros((3, 7)))
