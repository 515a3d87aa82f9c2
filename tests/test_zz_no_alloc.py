"""kqed_lattice_sum_noalloc, the lattice-sum entry point for callers that
cannot allocate GPU memory (codes whose own pool owns the device, loops where
cudaMalloc's implicit synchronisation would stall other streams): through the
C ABI it must give the results of kqed_lattice_sum_dev, on two calls in a row
(the static scratch keeps the previous call's contents), and reject a problem
whose scratch exceeds its fixed 16 MiB with a clear error.  Collected last, it
passes alone in a fresh process and after the other tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def setup():
    import torch

    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300 as K
    t = K.KernelTemps()
    yield K, t, torch
    t.free()


def _inputs(torch, L, a, nx, seed):
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_numpy
    ys = lattice_sites(L, a)
    xs = diagonal_x(nx, a)
    pi = pi_synth_numpy(xs, ys, seed=seed)
    dev = torch.device("cuda", 0)
    return (xs, ys, torch.as_tensor(xs, device=dev), torch.as_tensor(ys, device=dev),
            torch.as_tensor(pi, device=dev))


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_noalloc_matches_device_entry_point_twice(setup, variant):
    K, t, torch = setup
    xs, ys, dx, dy, dpi = _inputs(torch, 6, 0.25, 4, seed=21 + variant)
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
    K.lattice_sum_dev(t, variant, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), dpi.data_ptr(),
                      ref.data_ptr(), stream=stream)
    for _ in range(2):
        got = torch.full((len(xs),), float("nan"), dtype=torch.float64, device="cuda")
        K.lattice_sum_noalloc(t, variant, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys),
                              dpi.data_ptr(), got.data_ptr(), stream=stream)
        torch.cuda.synchronize()
        r = ref.cpu().numpy()
        g = got.cpu().numpy()
        assert np.all(np.isfinite(g))
        assert np.all(np.abs(g - r) <= TOL * np.maximum(np.abs(r), 1e-300) + 1e-300), (g, r)


def test_noalloc_second_call_with_other_inputs(setup):
    """a call after a call on different data must not see the old scratch"""
    K, t, torch = setup
    stream = torch.cuda.current_stream().cuda_stream
    for seed, L in [(31, 6), (32, 4)]:
        xs, ys, dx, dy, dpi = _inputs(torch, L, 0.3, 3, seed=seed)
        ref = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
        got = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
        K.lattice_sum_dev(t, 2, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), dpi.data_ptr(),
                          ref.data_ptr(), stream=stream)
        K.lattice_sum_noalloc(t, 2, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys),
                              dpi.data_ptr(), got.data_ptr(), stream=stream)
        torch.cuda.synchronize()
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        assert np.all(np.abs(g - r) <= TOL * np.maximum(np.abs(r), 1e-300) + 1e-300)


def test_noalloc_allocates_nothing(setup):
    """after a warm-up call (which loads the kernels' code), a call on a new
    problem size leaves the device's free memory unchanged"""
    K, t, torch = setup
    stream = torch.cuda.current_stream().cuda_stream
    xs, ys, dx, dy, dpi = _inputs(torch, 6, 0.25, 4, seed=41)
    got = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
    K.lattice_sum_noalloc(t, 3, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), dpi.data_ptr(),
                          got.data_ptr(), stream=stream)
    torch.cuda.synchronize()
    xs2, ys2, dx2, dy2, dpi2 = _inputs(torch, 5, 0.3, 3, seed=42)
    got2 = torch.zeros(len(xs2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    K.lattice_sum_noalloc(t, 3, dx2.data_ptr(), len(xs2), dy2.data_ptr(), len(ys2),
                          dpi2.data_ptr(), got2.data_ptr(), stream=stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert np.all(np.isfinite(got2.cpu().numpy()))


def test_noalloc_rejects_oversized_problem(setup):
    K, t, torch = setup
    ny = 20000   # L2 needs 388 * ny doubles of per-site terms: beyond 16 MiB
    dx = torch.zeros((2, 4), dtype=torch.float64, device="cuda")
    dy = torch.zeros((ny, 4), dtype=torch.float64, device="cuda")
    dpi = torch.zeros((1,), dtype=torch.float64, device="cuda")
    sums = torch.zeros(2, dtype=torch.float64, device="cuda")
    with pytest.raises(K.KQEDError, match="static limit"):
        K.lattice_sum_noalloc(t, 2, dx.data_ptr(), 2, dy.data_ptr(), ny, dpi.data_ptr(),
                              sums.data_ptr())
    # sizes whose scratch arithmetic would wrap are rejected before it is done
    with pytest.raises(K.KQEDError, match="static limit"):
        K.lattice_sum_noalloc(t, 2, dx.data_ptr(), 2, dy.data_ptr(), (1 << 62) + 1,
                              dpi.data_ptr(), sums.data_ptr())
