"""kqed_gb300 -- GB300-native evaluator of KQED's position-space QED kernel.

Python mirror of the reference C API over libkqed_gb300.so (include/kqed.h):

    t = KernelTemps()                  # initialise(&t): load + checksum + upload tables
    k = QED_kernel_L0(x, y, t)         # one pair, 384 doubles as [6][4][4][4]
    K = kernel_batch(t, 2, X, Y)       # many pairs, [n][384]
    s = lattice_sum(t, 2, X, Ysites, Pi)   # fused sum_y L(x,y).Pi(x,y) per x
    t.free()                           # free_QED_temps(&t)

All arithmetic runs in the CUDA library; there is no CPU fallback.  If the
library is missing the import of the binding raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkqed_gb300.so")

KQED_FP64, KQED_FP32_MIXED, KQED_SURROGATE = 0, 1, 2

# enum kqed_composite: the reference's composite kernels, by their function names
COMPOSITE_FUNCS = ["compute_all_kernels", "compute_all_Mkernels", "compute_all_Mkernels_v2",
                   "compute_con_kernels", "compute_con_kernels_v2", "compute_con_kernelsM_L2",
                   "compute_sub_kernelsM_L2", "compute_all_kernels_SYMXY",
                   "compute_all_kernels_SYMXY_v2", "compute_all_kernels_SYMXY0",
                   "compute_all_kernels_SYMXY0_v2"]
KQED_MKERNEL_L2 = 11
_COMPOSITE_WITH_M = ("compute_all_Mkernels", "compute_all_Mkernels_v2",
                     "compute_con_kernelsM_L2", "compute_sub_kernelsM_L2")
ST_OUT_OF_GRID, ST_TAYLOR_X, ST_SWAP, ST_AXIS = 1, 2, 4, 8


class AVX_precomps(ctypes.Structure):
    _fields_ = [("Fm", ctypes.c_void_p), ("Fp", ctypes.c_void_p), ("nmax", ctypes.c_int)]


class Grid_coeffs(ctypes.Structure):
    """struct Grid_coeffs, src/HEADERS/KQED.h:69-87 (layout unchanged)."""
    _fields_ = [
        ("Nffa", ctypes.c_int),
        ("Ffp", ctypes.c_void_p),
        ("Ffm", ctypes.c_void_p),
        ("XX", ctypes.POINTER(ctypes.c_double)),
        ("YY", ctypes.POINTER(ctypes.c_double)),
        ("xstp", ctypes.c_double),
        ("ystp", ctypes.c_double),
        ("nstpx", ctypes.c_int),
        ("nstpy", ctypes.c_int),
        ("TX", ctypes.POINTER(ctypes.POINTER(ctypes.c_double))),
        ("NtayX", ctypes.c_int),
        ("NY_tay", ctypes.c_int),
        ("TY", ctypes.POINTER(ctypes.POINTER(ctypes.c_double))),
        ("NtayY", ctypes.c_int),
        ("NX_tay", ctypes.c_int),
        ("PC", ctypes.POINTER(AVX_precomps)),
        ("nfx", ctypes.POINTER(ctypes.c_int)),
    ]


class QED_kernel_temps(ctypes.Structure):
    """struct QED_kernel_temps, src/HEADERS/KQED.h:90-93."""
    _fields_ = [("Grid", Grid_coeffs), ("G8", ctypes.POINTER(ctypes.c_int))]


_lib = None


class LatticeJob(ctypes.Structure):
    """struct kqed_lattice_job of include/kqed.h"""
    _fields_ = [("variant", ctypes.c_int), ("nx", ctypes.c_size_t), ("ny", ctypes.c_size_t),
                ("d_x", ctypes.c_void_p), ("d_y", ctypes.c_void_p), ("d_pi", ctypes.c_void_p),
                ("pi_seed", ctypes.c_uint64), ("pi_stream", ctypes.c_uint32),
                ("d_sums", ctypes.c_void_p)]


class BatchInfo(ctypes.Structure):
    """struct kqed_batch_info of include/kqed.h"""
    _fields_ = [("jobs", ctypes.c_int), ("units", ctypes.c_size_t), ("pairs", ctypes.c_size_t),
                ("warps_per_block", ctypes.c_int), ("blocks", ctypes.c_int),
                ("record_chunk_pairs", ctypes.c_size_t), ("graph_kernels", ctypes.c_size_t),
                ("tuned_ms", ctypes.c_double)]


class SurrogateOpts(ctypes.Structure):
    """struct kqed_surrogate_opts of include/kqed.h"""
    _fields_ = [("samples", ctypes.c_size_t), ("heldout", ctypes.c_size_t),
                ("batch", ctypes.c_int), ("epochs", ctypes.c_int), ("lr", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("tau", ctypes.c_double)]


class SurrogateReport(ctypes.Structure):
    """struct kqed_surrogate_report of include/kqed.h"""
    _fields_ = [(n, ctypes.c_double) for n in
                ("loss_final", "heldout_rms", "heldout_max", "untrained_rms", "untrained_max",
                 "train_seconds", "steps", "cells_accepted", "gemm_tflops", "seconds_total")]


def lib():
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libkqed_gb300.so not built: run `python -m kqed_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        T = ctypes.POINTER(QED_kernel_temps)
        L.initialise.argtypes = [T]
        L.initialise.restype = ctypes.c_int
        L.free_QED_temps.argtypes = [T]
        L.free_QED_temps.restype = None
        for v in range(4):
            f = getattr(L, "QED_kernel_L%d" % v)
            f.argtypes = [dp, dp, QED_kernel_temps, dp]
            f.restype = None
        L.kqed_kernel_batch.argtypes = [T, ctypes.c_int, ctypes.c_size_t, dp, dp, dp,
                                        ctypes.POINTER(ctypes.c_uint8), ctypes.c_int]
        L.kqed_kernel_batch.restype = ctypes.c_int
        L.kqed_kernel_batch_dev.argtypes = [T, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_void_p]
        L.kqed_kernel_batch_dev.restype = ctypes.c_int
        L.kqed_lattice_sum.argtypes = [T, ctypes.c_int, ctypes.c_size_t, dp, ctypes.c_size_t, dp,
                                       dp, dp, ctypes.c_int]
        L.kqed_lattice_sum.restype = ctypes.c_int
        L.kqed_lattice_sum_dev.argtypes = [T, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                           ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.kqed_lattice_sum_dev.restype = ctypes.c_int
        L.kqed_lattice_sum_noalloc.argtypes = [T, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                               ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]
        L.kqed_lattice_sum_noalloc.restype = ctypes.c_int
        L.kqed_last_error.restype = ctypes.c_char_p
        L.kqed_launch_count.restype = ctypes.c_uint64
        L.kqed_profile.argtypes = [ctypes.c_int]
        L.kqed_profile.restype = None
        L.kqed_profile_read.argtypes = [dp, ctypes.POINTER(ctypes.c_uint64)]
        L.kqed_profile_read.restype = ctypes.c_int
        L.kqed_profile_read_copies.argtypes = [dp, ctypes.POINTER(ctypes.c_uint64)]
        L.kqed_profile_read_copies.restype = ctypes.c_int
        L.kqed_precision_stats.argtypes = [T, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_double, dp, ctypes.c_void_p]
        L.kqed_precision_stats.restype = ctypes.c_int
        L.kqed_lattice_sum_synth.argtypes = [T, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                             ctypes.c_size_t, ctypes.c_void_p, ctypes.c_uint64,
                                             ctypes.c_uint32, ctypes.c_size_t, ctypes.c_size_t,
                                             ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.kqed_lattice_sum_synth.restype = ctypes.c_int
        L.kqed_pi_synth_dev.argtypes = [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p,
                                        ctypes.c_void_p]
        L.kqed_pi_synth_dev.restype = ctypes.c_int
        L.kqed_batch_plan_create.argtypes = [T, ctypes.c_int, ctypes.POINTER(LatticeJob),
                                             ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p)]
        L.kqed_batch_plan_create.restype = ctypes.c_int
        L.kqed_batch_plan_launch.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.kqed_batch_plan_launch.restype = ctypes.c_int
        L.kqed_batch_plan_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(BatchInfo)]
        L.kqed_batch_plan_info.restype = ctypes.c_int
        L.kqed_batch_plan_destroy.argtypes = [ctypes.c_void_p]
        L.kqed_batch_plan_destroy.restype = None
        L.kqed_bf16_gemm.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong,
                                     ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
        L.kqed_bf16_gemm.restype = ctypes.c_int
        T_ = ctypes.POINTER(QED_kernel_temps)
        L.kqed_surrogate_train.argtypes = [T_, ctypes.POINTER(SurrogateOpts),
                                           ctypes.POINTER(SurrogateReport)]
        L.kqed_surrogate_train.restype = ctypes.c_int
        L.kqed_surrogate_set_tolerance.argtypes = [T_, ctypes.c_double]
        L.kqed_surrogate_set_tolerance.restype = ctypes.c_int
        L.kqed_surrogate_served.argtypes = [T_, ctypes.POINTER(ctypes.c_uint64)]
        L.kqed_surrogate_served.restype = ctypes.c_int
        L.kqed_surrogate_cells.argtypes = [T_, ctypes.c_double, dp]
        L.kqed_surrogate_cells.restype = ctypes.c_int
        L.kqed_surrogate_weights.argtypes = [T_, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]
        L.kqed_surrogate_weights.restype = ctypes.c_int
        fp = ctypes.POINTER(ctypes.c_float)
        L.kqed_surrogate_export.argtypes = [T_, fp, fp]
        L.kqed_surrogate_export.restype = ctypes.c_int
        L.kqed_mlp_param_count.restype = ctypes.c_size_t
        L.kqed_mlp_forward_backward.argtypes = [fp, ctypes.c_size_t, fp, fp, fp, fp, dp]
        L.kqed_mlp_forward_backward.restype = ctypes.c_int
        L.kqed_mlp_infer.argtypes = [fp, ctypes.c_size_t, fp, fp]
        L.kqed_mlp_infer.restype = ctypes.c_int
        L.kqed_composite_size.argtypes = [ctypes.c_int]
        L.kqed_composite_size.restype = ctypes.c_size_t
        L.kqed_composite_batch.argtypes = [T, ctypes.c_int, dp, ctypes.c_size_t, dp, dp, dp,
                                           ctypes.c_int]
        L.kqed_composite_batch.restype = ctypes.c_int
        L.kqed_composite_batch_dev.argtypes = [T, ctypes.c_int, dp, ctypes.c_size_t,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_int, ctypes.c_void_p]
        L.kqed_composite_batch_dev.restype = ctypes.c_int
        for name in COMPOSITE_FUNCS:
            f = getattr(L, name)
            f.argtypes = ([dp] if name in _COMPOSITE_WITH_M else []) + [dp, dp, QED_kernel_temps,
                                                                        dp]
            f.restype = None
        L.QED_Mkernel_L2.argtypes = [ctypes.c_double, dp, dp, QED_kernel_temps, dp]
        L.QED_Mkernel_L2.restype = None
        L.kqed_pihat_batch.argtypes = [ctypes.c_size_t, dp, dp, dp]
        L.kqed_pihat_batch.restype = ctypes.c_int
        L.kqed_pihat_batch_dev.argtypes = [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p]
        L.kqed_pihat_batch_dev.restype = ctypes.c_int
        L.kqed_pihat_lattice_dev.argtypes = [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                             ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                             ctypes.c_void_p]
        L.kqed_pihat_lattice_dev.restype = ctypes.c_int
        L.ipihatFermLoop_antisym.argtypes = [dp, dp, QED_kernel_temps, dp]
        L.ipihatFermLoop_antisym.restype = None
        L.pihat1.argtypes = [dp, dp, QED_kernel_temps, dp, dp]
        L.pihat1.restype = None
        L.kqed_pinned_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
        L.kqed_pinned_alloc.restype = ctypes.c_int
        L.kqed_pinned_free.argtypes = [ctypes.c_void_p]
        L.kqed_pinned_free.restype = ctypes.c_int
        L.kqed_pinned_contains.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        L.kqed_pinned_contains.restype = ctypes.c_int
        L.kqed_fp32_peak_gflops.argtypes = [dp]
        L.kqed_fp32_peak_gflops.restype = ctypes.c_int
        L.kqed_fp64_peak_gflops.argtypes = [dp]
        L.kqed_fp64_peak_gflops.restype = ctypes.c_int
        _lib = L
    return _lib


class KQEDError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise KQEDError(lib().kqed_last_error().decode())


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _pairs(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a.reshape(1, 4)
    if a.ndim != 2 or a.shape[1] != 4:
        raise ValueError("expected 4-vectors, got shape %s" % (a.shape,))
    return a


class KernelTemps:
    """Owns a struct QED_kernel_temps; initialise() on construction
    (src/LIBFILES/init.c:142), free_QED_temps() on free()."""

    def __init__(self, lib_path=None):
        if lib_path is not None:
            os.environ["KQED_LIB_PATH"] = lib_path
        self.t = QED_kernel_temps()
        if lib().initialise(ctypes.byref(self.t)) != 0:
            raise KQEDError("initialise failed: " + lib().kqed_last_error().decode())

    @property
    def ptr(self):
        return ctypes.byref(self.t)

    def grid(self):
        g = self.t.Grid
        return {
            "nstpx": g.nstpx, "nstpy": g.nstpy,
            "XX": np.ctypeslib.as_array(g.XX, (g.nstpx,)).copy(),
            "YY": np.ctypeslib.as_array(g.YY, (g.nstpy,)).copy(),
            "nfx": np.ctypeslib.as_array(g.nfx, (g.nstpx,)).copy(),
        }

    def free(self):
        if self.t.Grid.PC:
            lib().free_QED_temps(ctypes.byref(self.t))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _legacy(v, x, y, t):
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(4)
    y = np.ascontiguousarray(y, dtype=np.float64).reshape(4)
    out = np.zeros((6, 4, 4, 4))
    getattr(lib(), "QED_kernel_L%d" % v)(_dptr(x), _dptr(y), t.t, _dptr(out))
    return out


def QED_kernel_L0(x, y, t):
    """QED_kernel_L0, src/LIBFILES/kernels.c:81-115."""
    return _legacy(0, x, y, t)


def QED_kernel_L1(x, y, t):
    """QED_kernel_L1, src/LIBFILES/kernels.c:117-134."""
    return _legacy(1, x, y, t)


def QED_kernel_L2(x, y, t):
    """QED_kernel_L2, src/LIBFILES/kernels.c:136-154."""
    return _legacy(2, x, y, t)


def QED_kernel_L3(x, y, t):
    """QED_kernel_L3, src/LIBFILES/kernels.c:156-177."""
    return _legacy(3, x, y, t)


def _out_array(out, shape):
    """the caller's output array (e.g. a PinnedArray's, which the kernels then
    write in place), checked, or a new one"""
    if out is None:
        return np.empty(shape)
    if out.shape != shape or out.dtype != np.float64 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float64 array of shape %s" % (shape,))
    return out


def kernel_batch(t, variant, x, y, precision=KQED_FP64, with_status=False, out=None):
    """L<variant>(x[i], y[i]) for all i: returns [n][384] (and [n] status bytes),
    in `out` if given."""
    x, y = _pairs(x), _pairs(y)
    if x.shape != y.shape:
        raise ValueError("x and y must have the same number of pairs")
    n = x.shape[0]
    out = _out_array(out, (n, 384))
    st = np.zeros(n, dtype=np.uint8) if with_status else None
    stp = st.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if with_status else None
    _check(lib().kqed_kernel_batch(t.ptr, variant, n, _dptr(x), _dptr(y), _dptr(out), stp,
                                   precision))
    return (out, st) if with_status else out


def kernel_batch_dev(t, variant, x_ptr, y_ptr, out_ptr, n, precision=KQED_FP64, status_ptr=None,
                     stream=None):
    """Device-pointer form (e.g. torch tensor .data_ptr()); enqueued on stream."""
    _check(lib().kqed_kernel_batch_dev(t.ptr, variant, n, x_ptr, y_ptr, out_ptr, status_ptr,
                                       precision, stream))


def composite_size(which):
    """doubles per pair of composite `which` (enum kqed_composite)"""
    return lib().kqed_composite_size(which)


def _masses(M):
    if M is None:
        return None
    return np.ascontiguousarray(np.atleast_1d(M), dtype=np.float64)


def composite_batch(t, which, x, y, M=None, precision=KQED_FP64, out=None):
    """Composite kernel `which` (enum kqed_composite) at every pair: returns
    [n][composite_size(which)] in the reference's struct layout, in `out` if
    given.  M: the four masses of the M-subtracted forms (one for
    QED_Mkernel_L2)."""
    x, y = _pairs(x), _pairs(y)
    if x.shape != y.shape:
        raise ValueError("x and y must have the same number of pairs")
    n = x.shape[0]
    out = _out_array(out, (n, composite_size(which)))
    Mv = _masses(M)
    _check(lib().kqed_composite_batch(t.ptr, which, None if Mv is None else _dptr(Mv), n,
                                      _dptr(x), _dptr(y), _dptr(out), precision))
    return out


def composite_batch_dev(t, which, x_ptr, y_ptr, out_ptr, n, M=None, precision=KQED_FP64,
                        stream=None):
    """Device-pointer form of composite_batch, enqueued on stream."""
    Mv = _masses(M)
    _check(lib().kqed_composite_batch_dev(t.ptr, which, None if Mv is None else _dptr(Mv), n,
                                          x_ptr, y_ptr, out_ptr, precision, stream))


def composite_call(name, x, y, t, M=None):
    """One pair through the reference-signature function `name` (e.g.
    "compute_con_kernelsM_L2", "QED_Mkernel_L2"); returns its output struct
    as a flat array."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(4)
    y = np.ascontiguousarray(y, dtype=np.float64).reshape(4)
    which = KQED_MKERNEL_L2 if name == "QED_Mkernel_L2" else COMPOSITE_FUNCS.index(name)
    out = np.zeros(composite_size(which))
    f = getattr(lib(), name)
    if name == "QED_Mkernel_L2":
        f(float(M), _dptr(x), _dptr(y), t.t, _dptr(out))
    elif name in _COMPOSITE_WITH_M:
        Mv = _masses(M)
        f(_dptr(Mv), _dptr(x), _dptr(y), t.t, _dptr(out))
    else:
        f(_dptr(x), _dptr(y), t.t, _dptr(out))
    return out


def pihat_batch(x, y):
    """ipihatFermLoop_antisym(x[i], y[i]) for all i: [n][384] (the reference's
    perturbative lepton-loop Pi-hat, src/LIBFILES/pi_pert.c)"""
    x, y = _pairs(x), _pairs(y)
    if x.shape != y.shape:
        raise ValueError("x and y must have the same number of pairs")
    out = np.empty((x.shape[0], 384))
    _check(lib().kqed_pihat_batch(x.shape[0], _dptr(x), _dptr(y), _dptr(out)))
    return out


def pihat_batch_dev(x_ptr, y_ptr, out_ptr, n, stream=None):
    _check(lib().kqed_pihat_batch_dev(n, x_ptr, y_ptr, out_ptr, stream))


def pihat_lattice_dev(x_ptr, nx, y_ptr, ny, scale, pi_ptr, stream=None):
    """pi[k][n][384] = Pi-hat(scale x_k, scale y_n), the fused sums' layout"""
    _check(lib().kqed_pihat_lattice_dev(nx, x_ptr, ny, y_ptr, scale, pi_ptr, stream))


def ipihatFermLoop_antisym(x, y, t):
    """ipihatFermLoop_antisym, src/LIBFILES/pi_pert.c:162-198 (one pair)"""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(4)
    y = np.ascontiguousarray(y, dtype=np.float64).reshape(4)
    out = np.zeros((6, 4, 4, 4))
    lib().ipihatFermLoop_antisym(_dptr(x), _dptr(y), t.t, _dptr(out))
    return out


def pihat1(x, y, t):
    """pihat1, src/LIBFILES/pi_pert.c:236-389: (vpihat1[4][4][4][4][4], vpihatr1[4][4][4][4])"""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(4)
    y = np.ascontiguousarray(y, dtype=np.float64).reshape(4)
    p = np.zeros((4, 4, 4, 4, 4))
    r = np.zeros((4, 4, 4, 4))
    lib().pihat1(_dptr(x), _dptr(y), t.t, _dptr(p), _dptr(r))
    return p, r


def pinned_contains(ptr, nbytes):
    """True if [ptr, ptr + nbytes) lies inside one kqed_pinned_alloc block
    (kqed_lattice_sum then reads a Pi there in place)."""
    return bool(lib().kqed_pinned_contains(ctypes.c_void_p(ptr), nbytes))


class PinnedArray:
    """A float64 array in page-locked, device-mapped host memory from
    kqed_pinned_alloc (cudaHostAlloc): `.array` is a numpy view of it; free()
    releases it.  kqed_lattice_sum reads a Pi held here in place."""

    def __init__(self, shape):
        self.shape = tuple(int(v) for v in np.atleast_1d(shape))
        n = int(np.prod(self.shape))
        self.ptr = ctypes.c_void_p()
        _check(lib().kqed_pinned_alloc(max(n, 1) * 8, ctypes.byref(self.ptr)))
        buf = (ctypes.c_double * max(n, 1)).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=np.float64, count=n).reshape(self.shape)

    def free(self):
        if self.ptr and self.ptr.value:
            self.array = None
            lib().kqed_pinned_free(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def lattice_sum(t, variant, x, ysites, pi, precision=KQED_FP64):
    """sums[k] = sum_n sum_c L<variant>_c(x_k, y_n) pi[k][n][c]."""
    x, ysites = _pairs(x), _pairs(ysites)
    pi = np.ascontiguousarray(pi, dtype=np.float64)
    if pi.shape != (x.shape[0], ysites.shape[0], 384):
        raise ValueError("pi must be [nx][ny][384]")
    sums = np.empty(x.shape[0])
    _check(lib().kqed_lattice_sum(t.ptr, variant, x.shape[0], _dptr(x), ysites.shape[0],
                                  _dptr(ysites), _dptr(pi), _dptr(sums), precision))
    return sums


def lattice_sum_dev(t, variant, x_ptr, nx, y_ptr, ny, pi_ptr, sums_ptr, precision=KQED_FP64,
                    stream=None):
    _check(lib().kqed_lattice_sum_dev(t.ptr, variant, nx, x_ptr, ny, y_ptr, pi_ptr, sums_ptr,
                                      precision, stream))


def lattice_sum_noalloc(t, variant, x_ptr, nx, y_ptr, ny, pi_ptr, sums_ptr, stream=None):
    """kqed_lattice_sum_noalloc: the device-pointer lattice sum with its scratch
    in a static 16 MiB device array (for callers that cannot allocate)."""
    _check(lib().kqed_lattice_sum_noalloc(t.ptr, variant, nx, x_ptr, ny, y_ptr, pi_ptr,
                                          sums_ptr, stream))


def launch_count():
    return int(lib().kqed_launch_count())


def profile(enable):
    """Start (True) or stop (False) event timing of the main kernels."""
    lib().kqed_profile(1 if enable else 0)


def lattice_sum_synth(t, variant, x_ptr, nx, y_ptr, ny, seed, sums_ptr, precision=KQED_FP64,
                      stream_id=0, x_offset=0, y_offset=0, stream=None):
    """Fused lattice sum with the synthetic Pi generated inside the kernel
    (kqed_lattice_sum_synth); device pointers.  x_offset / y_offset: global
    indices of the first x / site (a slab of a larger lattice)."""
    _check(lib().kqed_lattice_sum_synth(t.ptr, variant, nx, x_ptr, ny, y_ptr, seed, stream_id,
                                        x_offset, y_offset, sums_ptr, precision, stream))


def pi_synth_dev(x_ptr, nx, y_ptr, ny, seed, pi_ptr, stream_id=0, x_offset=0, y_offset=0,
                 stream=None):
    """The synthetic Pi of lattice_sum_synth written to pi_ptr [nx][ny][384]."""
    _check(lib().kqed_pi_synth_dev(nx, x_ptr, ny, y_ptr, seed, stream_id, x_offset, y_offset,
                                   pi_ptr, stream))


class BatchPlan:
    """A batch of fused lattice sums captured in one CUDA graph
    (kqed_batch_plan_*).  jobs: dicts with variant, nx, ny, d_x, d_y, d_pi
    (or None: generated Pi), pi_seed, pi_stream, d_sums (device pointers)."""

    def __init__(self, t, jobs, precision=KQED_FP64, tune=False):
        arr = (LatticeJob * len(jobs))()
        for i, j in enumerate(jobs):
            arr[i] = LatticeJob(j["variant"], j["nx"], j["ny"], j["d_x"], j["d_y"],
                                j.get("d_pi") or None, j.get("pi_seed", 0), j.get("pi_stream", 0),
                                j["d_sums"])
        self._h = ctypes.c_void_p()
        _check(lib().kqed_batch_plan_create(t.ptr, len(jobs), arr, precision, 1 if tune else 0,
                                            ctypes.byref(self._h)))

    def launch(self, stream=None):
        _check(lib().kqed_batch_plan_launch(self._h, stream))

    def info(self):
        i = BatchInfo()
        _check(lib().kqed_batch_plan_info(self._h, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in BatchInfo._fields_}

    def close(self):
        if self._h:
            lib().kqed_batch_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def precision_stats(t, variant, x_ptr, y_ptr, n, floor=1e-300, stream=None):
    """Error of the mixed form against the FP64 form of L<variant> on n device
    pairs, accumulated on the device (kqed_precision_stats): a dict with
    per-component max and RMS of the norm-relative error, the pair-level max
    and mean, and the number of pairs counted."""
    out = np.zeros(771)
    _check(lib().kqed_precision_stats(t.ptr, variant, n, x_ptr, y_ptr, floor, _dptr(out), stream))
    return {"comp_max": out[:384].copy(), "comp_rms": out[384:768].copy(),
            "pair_max": float(out[768]), "pair_mean": float(out[769]), "pairs": int(out[770])}


def profile_read():
    """(total milliseconds, launches) of the main kernels since profile(True)."""
    ms = ctypes.c_double()
    n = ctypes.c_uint64()
    _check(lib().kqed_profile_read(ctypes.byref(ms), ctypes.byref(n)))
    return ms.value, int(n.value)


def profile_read_copies():
    """(total milliseconds, copies) of the Pi chunk copies of lattice_sum."""
    ms = ctypes.c_double()
    n = ctypes.c_uint64()
    _check(lib().kqed_profile_read_copies(ctypes.byref(ms), ctypes.byref(n)))
    return ms.value, int(n.value)


def fp32_peak_gflops():
    g = ctypes.c_double()
    _check(lib().kqed_fp32_peak_gflops(ctypes.byref(g)))
    return g.value


def fp64_peak_gflops():
    g = ctypes.c_double()
    _check(lib().kqed_fp64_peak_gflops(ctypes.byref(g)))
    return g.value


def bf16_gemm(a_ptr, sam, sak, b_ptr, sbn, sbk, M, N, K, c_ptr, ldc, splits=1, stream=None):
    """kqed_bf16_gemm: c[z][m][n] = sum_k A(m,k) B(n,k) on the tensor cores
    (bf16 operands by strides, fp32 result); device pointers."""
    _check(lib().kqed_bf16_gemm(a_ptr, sam, sak, b_ptr, sbn, sbk, M, N, K, splits, c_ptr, ldc,
                                stream))


def surrogate_train(t, samples=10_000_000, heldout=1_000_000, batch=8192, epochs=4, lr=2e-3,
                    seed=5, tau=1e-3):
    """kqed_surrogate_train: train the weight-function network on the GPU and
    attach it to the tables (precision KQED_SURROGATE); returns the report."""
    o = SurrogateOpts(samples, heldout, batch, epochs, lr, seed, tau)
    r = SurrogateReport()
    _check(lib().kqed_surrogate_train(t.ptr, ctypes.byref(o), ctypes.byref(r)))
    return {f: getattr(r, f) for f, _ in SurrogateReport._fields_}


def surrogate_set_tolerance(t, tau):
    _check(lib().kqed_surrogate_set_tolerance(t.ptr, tau))


def surrogate_served(t):
    """pairs the network evaluated in lattice sums since the last call"""
    v = ctypes.c_uint64()
    _check(lib().kqed_surrogate_served(t.ptr, ctypes.byref(v)))
    return int(v.value)


def surrogate_cells(t, tau):
    """fraction of feature cells whose held-out error bound is <= tau"""
    v = ctypes.c_double()
    _check(lib().kqed_surrogate_cells(t.ptr, tau, ctypes.byref(v)))
    return v.value


def surrogate_weights(t, u_ptr, n, wnet_ptr, winterp_ptr=None, stream=None):
    """network (float [n][39]) and FP64 interpolation ([n][39]) weight functions
    at post-swap invariants u [n][3] = (|x|, |y|, cb); device pointers"""
    _check(lib().kqed_surrogate_weights(t.ptr, n, u_ptr, wnet_ptr, winterp_ptr, stream))


def mlp_param_count():
    return int(lib().kqed_mlp_param_count())


def surrogate_export(t):
    """(params [P] float32, norm [126] float32) of the attached network"""
    p = np.zeros(mlp_param_count(), dtype=np.float32)
    nm = np.zeros(9 + 3 * 39, dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    _check(lib().kqed_surrogate_export(t.ptr, p.ctypes.data_as(fp), nm.ctypes.data_as(fp)))
    return p, nm


def mlp_forward_backward(params, feat, target):
    """one forward/backward pass of the network on the GPU kernels: (y [n][39],
    grad [P], loss)"""
    params = np.ascontiguousarray(params, dtype=np.float32)
    feat = np.ascontiguousarray(feat, dtype=np.float32)
    target = np.ascontiguousarray(target, dtype=np.float32)
    n = feat.shape[0]
    y = np.zeros((n, 39), dtype=np.float32)
    g = np.zeros(mlp_param_count(), dtype=np.float32)
    loss = ctypes.c_double()
    fp = ctypes.POINTER(ctypes.c_float)
    _check(lib().kqed_mlp_forward_backward(params.ctypes.data_as(fp), n, feat.ctypes.data_as(fp),
                                           target.ctypes.data_as(fp), y.ctypes.data_as(fp),
                                           g.ctypes.data_as(fp), ctypes.byref(loss)))
    return y, g, loss.value


def mlp_infer(params, feat):
    """the network through the fused evaluation kernel: y [n][39]"""
    params = np.ascontiguousarray(params, dtype=np.float32)
    feat = np.ascontiguousarray(feat, dtype=np.float32)
    y = np.zeros((feat.shape[0], 39), dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    _check(lib().kqed_mlp_infer(params.ctypes.data_as(fp), feat.shape[0], feat.ctypes.data_as(fp),
                                y.ctypes.data_as(fp)))
    return y
