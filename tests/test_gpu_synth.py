"""Generated-Pi lattice sums (kqed_lattice_sum_synth, kqed_pi_synth_dev)
against the oracle's restatement of the generator and the stored-Pi entry
point.  Tolerances: generated Pi equal to the oracle's to 1e-15 relative
(the exponential of the envelope may differ in its last bit between the
device and the host C library); the fused sum with generated Pi equal bit
for bit to the stored-Pi sum over the same Pi written out; FP64 sums within
1e-12 of the oracle's contraction (relative to the largest |sum|)."""
import numpy as np
import pytest

from _helpers import oracle_contract, oracle_pi_synth

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


def _inputs():
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    ys = lattice_sites(6, 0.25)
    xs = np.vstack([diagonal_x(4, 0.25), [[0.3, -0.2, 0.5, 0.1]]])
    return xs, ys


def test_generated_pi_matches_oracle(temps):
    import torch
    xs, ys = _inputs()
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    pi = torch.empty((len(xs), len(ys), 384), dtype=torch.float64, device="cuda")
    K().pi_synth_dev(dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), 99, pi.data_ptr(),
                     stream_id=3)
    torch.cuda.synchronize()
    ref = oracle_pi_synth(xs, ys, 99, stream=3)
    got = pi.cpu().numpy()
    assert np.allclose(got, ref, rtol=1e-15, atol=0)


@pytest.mark.parametrize("variant", [0, 2, 3])
def test_lattice_sum_synth_equals_stored_pi_sum(temps, variant):
    import torch
    xs, ys = _inputs()
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    pi = torch.empty((len(xs), len(ys), 384), dtype=torch.float64, device="cuda")
    K().pi_synth_dev(dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), 5, pi.data_ptr())
    fp64 = None
    for prec in (K().KQED_FP64, K().KQED_FP32_MIXED):
        a = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
        b = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
        K().lattice_sum_dev(temps, variant, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys),
                            pi.data_ptr(), a.data_ptr(), prec)
        K().lattice_sum_synth(temps, variant, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys), 5,
                              b.data_ptr(), prec)
        torch.cuda.synchronize()
        assert np.array_equal(a.cpu().numpy(), b.cpu().numpy()), prec
        if fp64 is None:
            fp64 = a.cpu().numpy()
    ref = oracle_contract(variant, np.repeat(xs, len(ys), 0), np.tile(ys, (len(xs), 1)),
                          oracle_pi_synth(xs, ys, 5).reshape(-1, 384)).reshape(len(xs), -1).sum(1)
    assert np.abs(fp64 - ref).max() <= 1e-12 * np.abs(ref).max()


def test_site_slabs_with_offsets_reproduce_the_full_sum(temps):
    """the per-rank GPU evaluation of a sharded sum: slabs of sites with
    their global offsets, combined in rank order, give the whole lattice's
    generated-Pi sum (relative 1e-13)"""
    from kqed_gb300.shard import _gpu_local_sum, combine_rank_order, site_slab
    xs, ys = _inputs()
    full = _gpu_local_sum(temps, 2, xs, ys, 0, None, 17, 4, K().KQED_FP64)
    parts = []
    for r in range(3):
        lo, hi = site_slab(len(ys), r, 3)
        parts.append(_gpu_local_sum(temps, 2, xs, ys[lo:hi], lo, None, 17, 4, K().KQED_FP64))
    got = combine_rank_order(parts)
    assert np.abs(got - full).max() <= 1e-13 * np.abs(full).max()


def test_synth_lattice_workload_runs_small():
    """the large-lattice workload (generated Pi, both forms) on an 8^4
    lattice: one JSON line, FP64 checksum finite, mixed error within the
    1e-6 integrand bound at this size"""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-m", "benchmarks.synth_lattice_workload", "--L", "8",
                        "--nx", "4", "--steps", "1", "--warmup", "1"], cwd=root,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["evals_per_step"] == 4 * 8 ** 4
    assert np.isfinite(d["checksum_fp64"])
    assert d["fp32_mixed"]["err_vs_fp64"]["max"] <= 1e-6
    assert len(d["fp32_mixed"]["err_vs_fp64"]["per_x"]) == 4


def test_empty_lattice_sums_to_zero(temps):
    """an empty lattice (ny = 0; NULL site and Pi pointers) gives zero sums
    through every lattice entry point, in both forms"""
    import torch
    xs, _ = _inputs()
    nx = len(xs)
    dx = torch.as_tensor(xs, device="cuda")
    for prec in (K().KQED_FP64, K().KQED_FP32_MIXED):
        for v in (0, 2):
            out = torch.full((nx,), 7.0, dtype=torch.float64, device="cuda")
            K().lattice_sum_dev(temps, v, dx.data_ptr(), nx, 0, 0, 0, out.data_ptr(), prec)
            assert torch.count_nonzero(out).item() == 0
            out.fill_(7.0)
            K().lattice_sum_synth(temps, v, dx.data_ptr(), nx, 0, 0, 5, out.data_ptr(), prec)
            assert torch.count_nonzero(out).item() == 0
            h = K().lattice_sum(temps, v, xs, np.zeros((0, 4)), np.zeros((nx, 0, 384)), prec)
            assert np.array_equal(h, np.zeros(nx))
    out = torch.full((nx,), 7.0, dtype=torch.float64, device="cuda")
    K().lattice_sum_noalloc(temps, 2, dx.data_ptr(), nx, 0, 0, 0, out.data_ptr())
    torch.cuda.synchronize()
    assert torch.count_nonzero(out).item() == 0
