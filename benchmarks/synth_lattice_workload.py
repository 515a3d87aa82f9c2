"""Large fused lattice sums with generated Pi: sums[k] = sum_y L(x_k, y).Pi(x_k, y)
over a periodic L^4 lattice, Pi generated inside the kernels (seeded Philox,
the synthetic Pi of kqed_lattice_sum_synth), so that lattices whose stored
Pi would not fit in HBM (48^4 x 16 x: 261 GB) run at full size.

  python -m benchmarks.synth_lattice_workload [--L 48] [--nx 16] [--variant 2]

Default: 48^4 lattice, spacing 0.1, 16 diagonal x, kernel L2 -- 84,934,656
evaluations per step.  Both precision forms on the same inputs, timed with
CUDA events on the launching stream after warm-up; the mixed form's
integrand error against the FP64 sums of the same run
(|S_mixed - S_fp64| / rms_x(S_fp64)).  Prints one JSON line.
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--L", type=int, default=48)
    p.add_argument("--spacing", type=float, default=0.1)
    p.add_argument("--nx", type=int, default=16)
    p.add_argument("--variant", type=int, default=2)
    p.add_argument("--seed", type=int, default=11)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    a = p.parse_args()
    sys.path.insert(0, ROOT)
    import torch

    import kqed_gb300 as K
    from benchmarks.clocks import ClockSampler
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    t = K.KernelTemps()
    xs = diagonal_x(a.nx, a.spacing)
    ys = lattice_sites(a.L, a.spacing)
    nx, ny = len(xs), len(ys)
    dx = torch.as_tensor(xs, device="cuda")
    dy = torch.as_tensor(ys, device="cuda")
    stream = torch.cuda.current_stream()
    res, sums = {}, {}
    for name, prec in (("fp64", K.KQED_FP64), ("fp32_mixed", K.KQED_FP32_MIXED)):
        out = torch.zeros(nx, dtype=torch.float64, device="cuda")

        def step():
            K.lattice_sum_synth(t, a.variant, dx.data_ptr(), nx, dy.data_ptr(), ny, a.seed,
                                out.data_ptr(), prec, stream=stream.cuda_stream)
        clk = ClockSampler(torch.cuda.current_device())
        clk.start()
        for _ in range(a.warmup):
            step()
        torch.cuda.synchronize()
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
        res[name] = {"ms_per_step": ms, "evals_per_s": nx * ny / (ms / 1e3), "clocks": clocks}
    s64, s32 = sums["fp64"], sums["fp32_mixed"]
    rms = float(np.sqrt(np.mean(s64 ** 2)))
    err = np.abs(s32 - s64) / rms
    res["fp32_mixed"].update({
        "speedup_vs_fp64": res["fp64"]["ms_per_step"] / res["fp32_mixed"]["ms_per_step"],
        "err_vs_fp64": {"definition": "per x: |S_fp32 - S_fp64| / rms_x(S_fp64)",
                        "max": float(err.max()), "median": float(np.median(err)),
                        "per_x": [float("%.3g" % e) for e in err]}})
    print(json.dumps({
        "workload": "fused lattice sum, kernel L%d, periodic %d^4 lattice, spacing %g, %d x "
                    "points on the diagonal, generated Pi (seed %d)"
                    % (a.variant, a.L, a.spacing, nx, a.seed),
        "evals_per_step": nx * ny, "checksum_fp64": float(np.sum(s64)), **res}))
    t.free()


if __name__ == "__main__":
    main()
