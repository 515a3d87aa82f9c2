"""Batched-lattice workload: many fused lattice sums in one CUDA graph.

  python -m benchmarks.batch_workload [--jobs 64] [--seed 3] [--steps 3]

Jobs: lattice size L and kernel variant drawn (numpy default_rng(seed)) from
{12, 16, 24, 32} x {L0, L1, L2, L3}; every job is a periodic L^4 lattice
with spacing 0.1 and 8 points x_k = 0.1 k (1,1,1,1), k = 0..7; Pi is the
generated synthetic Pi (key = seed, counter stream = job index), so no Pi is
stored.  Sites of equal L share one device array (and so their per-site
kernel terms).

For each precision form the batch is planned with the autotuner and the
CUDA graph replayed --steps times (timed with CUDA events); the same jobs
run one after another through kqed_lattice_sum_synth (no graph, no work
list) for comparison, and the two results are checked against each other.
Prints one JSON line.
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def make_jobs(njobs, seed):
    rng = np.random.default_rng(seed)
    Ls = rng.choice([12, 16, 24, 32], size=njobs)
    vs = rng.integers(0, 4, size=njobs)
    return [(int(L), int(v)) for L, v in zip(Ls, vs)]


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--jobs", type=int, default=64)
    p.add_argument("--seed", type=int, default=3)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--nx", type=int, default=8)
    a = p.parse_args()
    sys.path.insert(0, ROOT)
    import torch

    import kqed_gb300 as K
    from benchmarks.clocks import ClockSampler
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    t = K.KernelTemps()
    specs = make_jobs(a.jobs, a.seed)
    sites = {L: torch.as_tensor(lattice_sites(L, 0.1), device="cuda")
             for L in sorted(set(L for L, _ in specs))}
    dx = torch.as_tensor(diagonal_x(a.nx, 0.1), device="cuda")
    pairs = sum(a.nx * len(sites[L]) for L, _ in specs)
    out = {"workload": "%d lattices, L and variant drawn (seed %d) from {12,16,24,32} x {L0..L3}, "
                       "%d diagonal x each, spacing 0.1, generated Pi" % (a.jobs, a.seed, a.nx),
           "pairs_per_step": pairs,
           "jobs_by_L": {str(L): sum(1 for q, _ in specs if q == L) for L in sites}}
    for name, prec in (("fp64", K.KQED_FP64), ("fp32_mixed", K.KQED_FP32_MIXED)):
        sums = [torch.zeros(a.nx, dtype=torch.float64, device="cuda") for _ in specs]
        jobs = [{"variant": v, "nx": a.nx, "ny": len(sites[L]), "d_x": dx.data_ptr(),
                 "d_y": sites[L].data_ptr(), "d_pi": None, "pi_seed": a.seed, "pi_stream": j,
                 "d_sums": sums[j].data_ptr()} for j, (L, v) in enumerate(specs)]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        plan = K.BatchPlan(t, jobs, precision=prec, tune=True)
        e1.record()
        torch.cuda.synchronize()
        plan_ms = e0.elapsed_time(e1)
        clk = ClockSampler(torch.cuda.current_device())
        clk.start()
        plan.launch()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(a.steps):
            plan.launch()
        e1.record()
        torch.cuda.synchronize()
        clocks = clk.stop()
        graph_ms = e0.elapsed_time(e1) / a.steps
        got = np.concatenate([s.cpu().numpy() for s in sums])
        # the same jobs, one call each
        ref = [torch.zeros(a.nx, dtype=torch.float64, device="cuda") for _ in specs]
        e0.record()
        for j, (L, v) in enumerate(specs):
            K.lattice_sum_synth(t, v, dx.data_ptr(), a.nx, sites[L].data_ptr(), len(sites[L]),
                                a.seed, ref[j].data_ptr(), prec, stream_id=j)
        e1.record()
        torch.cuda.synchronize()
        seq_ms = e0.elapsed_time(e1)
        r = np.concatenate([s.cpu().numpy() for s in ref])
        info = plan.info()
        out[name] = {"graph_ms_per_step": graph_ms, "evals_per_s": pairs / (graph_ms / 1e3),
                     "sequential_calls_ms": seq_ms,
                     "sequential_evals_per_s": pairs / (seq_ms / 1e3),
                     "plan_create_ms": plan_ms, "clocks": clocks,
                     "max_rel_diff_vs_sequential": float(np.abs(got - r).max() /
                                                         max(np.abs(r).max(), 1e-300)),
                     "launch": {k: info[k] for k in ("warps_per_block", "blocks",
                                                     "record_chunk_pairs", "graph_kernels",
                                                     "tuned_ms")}}
        plan.close()
    print(json.dumps(out))
    t.free()


if __name__ == "__main__":
    main()
