"""Host buffers in kqed_pinned_alloc memory, which the kernels use in place:
kqed_lattice_sum's Pi (read over the host link; other memory, or
KQED_HOST_PI=copy, is staged through device buffers) and the outputs of
kqed_kernel_batch and kqed_composite_batch (written in place).  Each route
must give the same results bit for bit, in both precision forms."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def temps():
    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300 as K
    t = K.KernelTemps()
    yield t
    t.free()


def K():
    import kqed_gb300
    return kqed_gb300


def _case():
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_numpy
    xs = diagonal_x(5, 0.1)
    ys = np.ascontiguousarray(lattice_sites(10, 0.1)[::3])
    return xs, ys, pi_synth_numpy(xs, ys, seed=91)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pinned_pi_read_in_place_equals_staged_copies(temps, precision, monkeypatch):
    prec = K().KQED_FP64 if precision == "fp64" else K().KQED_FP32_MIXED
    xs, ys, pi = _case()
    staged = K().lattice_sum(temps, 2, xs, ys, pi, precision=prec)   # pageable: copies
    buf = K().PinnedArray((pi.size + 1000,))
    try:
        # a sub-range of the block, not at its start
        view = buf.array[500:500 + pi.size].reshape(pi.shape)
        view[...] = pi
        assert K().pinned_contains(view.ctypes.data, view.nbytes)
        in_place = K().lattice_sum(temps, 2, xs, ys, view, precision=prec)
        assert np.array_equal(in_place, staged)
        monkeypatch.setenv("KQED_HOST_PI", "copy")
        forced = K().lattice_sum(temps, 2, xs, ys, view, precision=prec)
        assert np.array_equal(forced, staged)
    finally:
        buf.free()


def test_pinned_range_check(temps):
    buf = K().PinnedArray((1024,))
    try:
        p = buf.array.ctypes.data
        assert K().pinned_contains(p, 1024 * 8)
        assert K().pinned_contains(p + 8, 1023 * 8)
        assert not K().pinned_contains(p + 8, 1024 * 8)      # one double past the end
        assert not K().pinned_contains(p, 0)
    finally:
        buf.free()
    assert not K().pinned_contains(p, 8)                     # freed
    a = np.zeros(16)
    assert not K().pinned_contains(a.ctypes.data, a.nbytes)  # pageable memory


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_in_place_pipeline_over_several_record_passes(temps, precision):
    """60 x against 20,000 sites: more pairs than one record pass holds, so
    the in-place route alternates x chunks between its two streams and
    record buffers; the sums equal the device path's bit for bit"""
    import torch
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_torch
    prec = K().KQED_FP64 if precision == "fp64" else K().KQED_FP32_MIXED
    xs = diagonal_x(60, 0.1)
    ys = np.ascontiguousarray(lattice_sites(24, 0.1)[::16][:20000])
    pi = pi_synth_torch(xs, ys, seed=93)                     # 3.7 GB on the device
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    dev = torch.empty(len(xs), dtype=torch.float64, device="cuda")
    K().lattice_sum_dev(temps, 2, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), pi.data_ptr(),
                        dev.data_ptr(), prec, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ref = dev.cpu().numpy()
    buf = K().PinnedArray(tuple(pi.shape))
    try:
        torch.from_numpy(buf.array).copy_(pi)
        del pi
        torch.cuda.empty_cache()
        assert K().pinned_contains(buf.array.ctypes.data, buf.array.nbytes)
        got = K().lattice_sum(temps, 2, xs, ys, buf.array, precision=prec)
        assert np.array_equal(got, ref)
    finally:
        buf.free()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_pair_batch_output_in_place(temps, variant, precision):
    """kqed_kernel_batch writes an output in kqed_pinned_alloc memory in
    place: the same values and status bytes as through a device buffer"""
    from kqed_gb300.workloads import config1_pairs
    prec = K().KQED_FP64 if precision == "fp64" else K().KQED_FP32_MIXED
    x, y = config1_pairs()
    x = np.vstack([x, np.zeros((1, 4)), y[:1]])     # x = 0 and x = y rows
    y = np.vstack([y, y[:1], y[:1]])
    ref, st_ref = K().kernel_batch(temps, variant, x, y, precision=prec, with_status=True)
    buf = K().PinnedArray((len(x), 384))
    try:
        got, st = K().kernel_batch(temps, variant, x, y, precision=prec, with_status=True,
                                   out=buf.array)
        assert got is buf.array
        assert np.array_equal(got, ref) and np.array_equal(st, st_ref)
    finally:
        buf.free()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("which", [0, 5])
def test_composite_output_in_place(temps, which, precision):
    """kqed_composite_batch writes an output in kqed_pinned_alloc memory in
    place (one pass over all pairs): the same values as through staging"""
    prec = K().KQED_FP64 if precision == "fp64" else K().KQED_FP32_MIXED
    rng = np.random.default_rng(which + 5)
    n = 40000                                        # more than one launch group
    x = rng.uniform(-2, 2, (n, 4))
    y = rng.uniform(-2, 2, (n, 4))
    M = [0.0, 0.5, 1.0, 1.5]
    ref = K().composite_batch(temps, which, x, y, M=M, precision=prec)
    buf = K().PinnedArray(ref.shape)
    try:
        got = K().composite_batch(temps, which, x, y, M=M, precision=prec, out=buf.array)
        assert np.array_equal(got, ref)
    finally:
        buf.free()
