"""The learned surrogate end to end on one GPU: training, then the lattice
sum it serves.

  python -m benchmarks.surrogate_workload [--samples 1e7] [--epochs 4] [--L 48] [--nx 16]

1. Train the weight-function network on the GPU (kqed_surrogate_train):
   |x|, |y| log-uniform over the form-factor grid, cb uniform on [-1, 1],
   labels from the FP64 interpolation, 10 % more samples held out for the
   per-cell error bounds.  Reported: training time, tensor-core rate,
   held-out error of the trained and of the untrained network.
2. The fused lattice sum with generated Pi (kqed_lattice_sum_synth) on a
   periodic L^4 lattice, spacing 0.1, nx points on the (1,1,1,1) diagonal,
   kernel L2 -- default 48^4 x 16 x = 84,934,656 evaluations per step --
   in the FP64 form, the mixed form, and the surrogate form at several
   acceptance bounds tau (in units of the weight functions' local scale):
   evaluations/s with CUDA events after warm-up, the share of pairs the
   network evaluated, and the integrand error against the FP64 sums
   (per x |S - S_fp64| / rms_x(S_fp64)).  tau = 0 is the fallback-only
   path (the mixed form's interpolation everywhere).
Prints one JSON line.
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--samples", type=float, default=1e7)
    p.add_argument("--heldout", type=float, default=1e6)
    p.add_argument("--epochs", type=int, default=4)
    p.add_argument("--batch", type=int, default=8192)
    p.add_argument("--lr", type=float, default=2e-3)
    p.add_argument("--L", type=int, default=48)
    p.add_argument("--spacing", type=float, default=0.1)
    p.add_argument("--nx", type=int, default=16)
    p.add_argument("--variant", type=int, default=2)
    p.add_argument("--seed", type=int, default=11)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=2)
    p.add_argument("--taus", default="0,0.01,0.03,0.1,inf")
    a = p.parse_args()
    sys.path.insert(0, ROOT)
    import torch

    import kqed_gb300 as K
    from benchmarks.clocks import ClockSampler
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    t = K.KernelTemps()
    train = K.surrogate_train(t, samples=int(a.samples), heldout=int(a.heldout), batch=a.batch,
                              epochs=a.epochs, lr=a.lr, seed=5, tau=0.0)
    xs = diagonal_x(a.nx, a.spacing)
    ys = lattice_sites(a.L, a.spacing)
    nx, ny = len(xs), len(ys)
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    stream = torch.cuda.current_stream()
    forms = [("fp64", K.KQED_FP64, None), ("fp32_mixed", K.KQED_FP32_MIXED, None)]
    for tau in a.taus.split(","):
        forms.append(("surrogate_tau_%s" % tau, K.KQED_SURROGATE, float(tau)))
    res, sums = {}, {}
    for name, prec, tau in forms:
        if tau is not None:
            K.surrogate_set_tolerance(t, tau)
        out = torch.zeros(nx, dtype=torch.float64, device="cuda")

        def step():
            K.lattice_sum_synth(t, a.variant, dx.data_ptr(), nx, dy.data_ptr(), ny, a.seed,
                                out.data_ptr(), prec, stream=stream.cuda_stream)
        for _ in range(a.warmup):
            step()
        torch.cuda.synchronize()
        if tau is not None:
            K.surrogate_served(t)
        clk = ClockSampler(torch.cuda.current_device())
        clk.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        clocks = clk.stop()
        ms = e0.elapsed_time(e1) / a.steps
        sums[name] = out.cpu().numpy()
        r = {"ms_per_step": ms, "evals_per_s": nx * ny / (ms / 1e3), "clocks": clocks}
        if tau is not None:
            r["tau"] = tau
            r["cells_accepted"] = K.surrogate_cells(t, tau)
            r["network_share"] = K.surrogate_served(t) / (a.steps * nx * ny)
        res[name] = r
    s64 = sums["fp64"]
    rms = float(np.sqrt(np.mean(s64 ** 2)))
    for name, _, _ in forms[1:]:
        err = np.abs(sums[name] - s64) / rms
        res[name].update({
            "speedup_vs_fp64": res["fp64"]["ms_per_step"] / res[name]["ms_per_step"],
            "err_vs_fp64": {"max": float(err.max()), "median": float(np.median(err))}})
    print(json.dumps({
        "workload": "fused lattice sum, kernel L%d, periodic %d^4 lattice, spacing %g, %d x "
                    "points on the diagonal, generated Pi (seed %d)"
                    % (a.variant, a.L, a.spacing, nx, a.seed),
        "err_definition": "per x: |S - S_fp64| / rms_x(S_fp64)",
        "evals_per_step": nx * ny, "training": train, **res}))
    t.free()


if __name__ == "__main__":
    main()
