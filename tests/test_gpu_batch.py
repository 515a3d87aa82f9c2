"""Batched lattices in one CUDA graph (kqed_batch_plan_*): every job's sums
equal the single-lattice entry points' on the same inputs (relative 1e-13:
the batch may choose a different assembly block shape, which reorders the
compensated per-tile sums), replays are bit-for-bit repeatable, and the
tuned plan agrees with the untuned one to the same tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-13


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


def _jobs(torch):
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    specs = [(4, 0, True), (5, 1, False), (4, 2, True), (6, 3, True), (5, 2, False), (4, 3, False)]
    sites = {L: torch.as_tensor(lattice_sites(L, 0.2), device="cuda") for L in (4, 5, 6)}
    jobs, keep = [], []
    for i, (L, v, gen) in enumerate(specs):
        xs = diagonal_x(3, 0.2) + 0.05 * i
        dx = torch.as_tensor(xs, device="cuda")
        dy = sites[L]
        sums = torch.zeros(len(xs), dtype=torch.float64, device="cuda")
        pi = None
        if not gen:
            pi = torch.empty((len(xs), len(dy), 384), dtype=torch.float64, device="cuda")
            K().pi_synth_dev(dx.data_ptr(), len(xs), dy.data_ptr(), len(dy), 100 + i,
                             pi.data_ptr(), stream_id=i)
        jobs.append({"variant": v, "nx": len(xs), "ny": len(dy), "d_x": dx.data_ptr(),
                     "d_y": dy.data_ptr(), "d_pi": pi.data_ptr() if pi is not None else None,
                     "pi_seed": 100 + i, "pi_stream": i, "d_sums": sums.data_ptr()})
        keep.append((dx, dy, sums, pi))
    return jobs, keep


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_plan_matches_single_lattice_calls(temps, precision):
    import torch
    jobs, keep = _jobs(torch)
    plan = K().BatchPlan(temps, jobs, precision=precision)
    plan.launch()
    torch.cuda.synchronize()
    got = [k[2].cpu().numpy().copy() for k in keep]
    plan.launch()
    torch.cuda.synchronize()
    for g, k in zip(got, keep):
        assert np.array_equal(g, k[2].cpu().numpy())
    info = plan.info()
    assert info["jobs"] == len(jobs) and info["graph_kernels"] > 0
    for j, (dx, dy, sums, pi) in zip(jobs, keep):
        ref = torch.zeros_like(sums)
        if pi is None:
            K().lattice_sum_synth(temps, j["variant"], dx.data_ptr(), j["nx"], dy.data_ptr(),
                                  j["ny"], j["pi_seed"], ref.data_ptr(), precision,
                                  stream_id=j["pi_stream"])
        else:
            K().lattice_sum_dev(temps, j["variant"], dx.data_ptr(), j["nx"], dy.data_ptr(),
                                j["ny"], pi.data_ptr(), ref.data_ptr(), precision)
        torch.cuda.synchronize()
        r = ref.cpu().numpy()
        g = sums.cpu().numpy()
        assert np.abs(g - r).max() <= REL * np.abs(r).max(), (j["variant"], g, r)
    plan.close()


def test_tuned_batch_plan(temps):
    import torch
    jobs, keep = _jobs(torch)
    plan = K().BatchPlan(temps, jobs, precision=0)
    plan.launch()
    torch.cuda.synchronize()
    base = [k[2].cpu().numpy().copy() for k in keep]
    plan.close()
    tuned = K().BatchPlan(temps, jobs, precision=0, tune=True)
    info = tuned.info()
    assert info["tuned_ms"] > 0 and info["warps_per_block"] in (2, 4)
    tuned.launch()
    torch.cuda.synchronize()
    for b, k in zip(base, keep):
        g = k[2].cpu().numpy()
        assert np.abs(g - b).max() <= REL * np.abs(b).max()
    tuned.close()


@pytest.mark.parametrize("precision", [0])
def test_batch_jobs_match_oracle(temps, precision):
    """jobs of the batch (stored and generated Pi, L0..L3) against the
    oracle's contraction: |S - S_oracle| <= 1e-12 * sum_y |L.Pi|"""
    import torch

    from _helpers import oracle_contract, oracle_pi_synth
    jobs, keep = _jobs(torch)
    plan = K().BatchPlan(temps, jobs, precision=precision)
    plan.launch()
    torch.cuda.synchronize()
    for j, (dx, dy, sums, pi) in list(zip(jobs, keep))[:4]:
        xs, ys = dx.cpu().numpy(), dy.cpu().numpy()
        if pi is None:
            P = oracle_pi_synth(xs, ys, j["pi_seed"], j["pi_stream"])
        else:
            P = pi.cpu().numpy()
        g = sums.cpu().numpy()
        for k in range(len(xs)):
            X = np.repeat(xs[k:k + 1], len(ys), 0)
            terms = oracle_contract(j["variant"], X, ys, P[k])
            assert abs(g[k] - np.sum(terms)) <= 1e-12 * np.sum(np.abs(terms)), (j["variant"], k)
    plan.close()
