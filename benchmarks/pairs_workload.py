"""Non-fused pair batches: L<variant>(x_i, y_i), 384 FP64 components each.

  python -m benchmarks.pairs_workload [--variant 0] [--repeat 64] [--steps 5]

Pairs: the 4160 pairs of workloads.config1_pairs (4096 with components
U[-2,2], 64 with one side of norm 1e-6..1e-3), tiled `--repeat` times so
that one launch keeps the GPU busy; device-resident inputs and outputs,
timed with CUDA events, clocks sampled.  Both precision forms, with the mixed form's
per-pair norm-relative error against the FP64 form.  Prints one JSON line.
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--variant", type=int, default=0)
    p.add_argument("--repeat", type=int, default=64)
    p.add_argument("--steps", type=int, default=5)
    a = p.parse_args()
    sys.path.insert(0, ROOT)
    import torch

    import kqed_gb300 as K
    from benchmarks.clocks import ClockSampler
    from kqed_gb300.workloads import config1_pairs
    t = K.KernelTemps()
    x, y = config1_pairs()
    x = np.tile(x, (a.repeat, 1))
    y = np.tile(y, (a.repeat, 1))
    n = len(x)
    dx = torch.as_tensor(x, device="cuda")
    dy = torch.as_tensor(y, device="cuda")
    out = {}
    res = {}
    for name, prec in (("fp64", K.KQED_FP64), ("fp32_mixed", K.KQED_FP32_MIXED)):
        o = torch.empty((n, 384), dtype=torch.float64, device="cuda")
        for _ in range(2):
            K.kernel_batch_dev(t, a.variant, dx.data_ptr(), dy.data_ptr(), o.data_ptr(), n, prec)
        torch.cuda.synchronize()
        clk = ClockSampler(torch.cuda.current_device())
        clk.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.steps):
            K.kernel_batch_dev(t, a.variant, dx.data_ptr(), dy.data_ptr(), o.data_ptr(), n, prec)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.steps
        res[name] = o
        out[name] = {"ms_per_step": ms, "evals_per_s": n / (ms / 1e3), "clocks": clk.stop()}
    a64, a32 = res["fp64"], res["fp32_mixed"]
    nrm = a64.abs().max(1).values
    live = nrm > 0
    err = ((a32 - a64).abs().max(1).values[live] / nrm[live]).cpu().numpy()
    out["fp32_mixed"].update({"speedup_vs_fp64": out["fp64"]["ms_per_step"] /
                              out["fp32_mixed"]["ms_per_step"],
                              "pair_err_max": float(err.max()),
                              "pair_err_median": float(np.median(err))})
    print(json.dumps({"workload": "L%d on %d pairs (the 4160 config-1 pairs x %d), output "
                                  "[n][384] FP64" % (a.variant, n, a.repeat), **out}))
    t.free()


if __name__ == "__main__":
    main()
