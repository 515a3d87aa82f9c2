"""The perturbative lepton-loop Pi-hat on one GPU, and the lepton-loop
lattice integrand it feeds.

  python -m benchmarks.pihat_workload [--n 65536] [--L 16] [--nx 4]

1. ipihatFermLoop_antisym over --n seeded pairs (components U[-2,2]),
   device-resident (kqed_pihat_batch_dev): pairs/s with CUDA events after
   warm-up; the CPU oracle (the reference's algorithm, all host cores) on a
   bounded sample; parity of the sample.
2. The lepton-loop integrand of the reference's a_mu check
   (src/amu_forlattice.c:65-116) on a periodic L^4 lattice at spacing 0.1,
   its sites shifted by half a spacing in every direction (the massive
   propagators are singular at y = 0 and y = x, which the reference's own
   check avoids), with nx points on the diagonal from x = 0.1 (1,1,1,1) on:
   Pi-hat(Mv x, Mv y), Mv = 2, generated in
   the fused sums' layout (kqed_pihat_lattice_dev), then the fused FP64
   lattice sum of L0 against it (kqed_lattice_sum_dev); the time of each.
Prints one JSON line.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=65536)
    p.add_argument("--L", type=int, default=16)
    p.add_argument("--nx", type=int, default=4)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--cpu-pairs", type=int, default=256)
    a = p.parse_args()
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch

    import kqed_gb300 as K
    from _helpers import oracle_pihat
    from benchmarks.clocks import ClockSampler
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    t = K.KernelTemps()
    rng = np.random.default_rng(5)
    x = rng.uniform(-2, 2, (a.n, 4))
    y = rng.uniform(-2, 2, (a.n, 4))
    dx = torch.as_tensor(x, device="cuda")
    dy = torch.as_tensor(y, device="cuda")
    out = torch.empty((a.n, 384), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()

    def step():
        K.pihat_batch_dev(dx.data_ptr(), dy.data_ptr(), out.data_ptr(), a.n, s.cuda_stream)
    step()
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(a.steps):
        step()
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    res = {"pairs": {"n": a.n, "ms_per_step": ms, "pairs_per_s": a.n / (ms / 1e3),
                     "clocks": clk.stop()}}
    m = min(a.cpu_pairs, a.n)
    t0 = time.perf_counter()
    ref = oracle_pihat(x[:m], y[:m])
    dt = time.perf_counter() - t0
    got = out[:m].cpu().numpy()
    d = (np.abs(got - ref).max(1) / np.abs(ref).max(1)).max()
    res["pairs"]["cpu"] = {"pairs_per_s": m / dt, "kind": "port", "cores": os.cpu_count(),
                           "sample": "first %d pairs" % m}
    res["pairs"]["parity"] = {"max_rel": float(d), "tol": 1e-12, "ok": bool(d <= 1e-12)}
    # the lepton-loop integrand on a lattice
    xs = diagonal_x(a.nx + 1, 0.1)[1:]   # x = 0 is singular for Pi-hat
    ys = lattice_sites(a.L, 0.1) + 0.05
    nx, ny = len(xs), len(ys)
    gx = torch.as_tensor(xs, device="cuda")
    gy = torch.as_tensor(ys, device="cuda")
    pi = torch.empty((nx, ny, 384), dtype=torch.float64, device="cuda")
    sums = torch.empty(nx, dtype=torch.float64, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    for rep in range(2):
        ev[0].record(s)
        K.pihat_lattice_dev(gx.data_ptr(), nx, gy.data_ptr(), ny, 2.0, pi.data_ptr(), s.cuda_stream)
        ev[1].record(s)
        K.lattice_sum_dev(t, 0, gx.data_ptr(), nx, gy.data_ptr(), ny, pi.data_ptr(),
                          sums.data_ptr(), K.KQED_FP64, s.cuda_stream)
        ev[2].record(s)
        torch.cuda.synchronize()
    res["lepton_loop_lattice"] = {
        "workload": "periodic %d^4 lattice, spacing 0.1, sites shifted by (0.05,0.05,0.05,0.05), "
                    "%d x on the diagonal, L0 . Pi-hat(2x, 2y)" % (a.L, nx),
        "pairs": nx * ny, "pihat_ms": ev[0].elapsed_time(ev[1]),
        "lattice_sum_ms": ev[1].elapsed_time(ev[2]), "sums": sums.cpu().tolist()}
    print(json.dumps(res))
    t.free()


if __name__ == "__main__":
    main()
