"""Error statistics of the mixed-precision form against the FP64 form on a
large random pair set, accumulated on the device (kqed_precision_stats).

  python -m benchmarks.stats_workload [--pairs 1e8] [--variant 3] [--seed 4]

Pairs: x, y uniform in [-4, 4]^4; 1% of them get a small side: |x| (half of
them) or |y| (the other half) scaled into [1e-4, 1e-2) (log-uniform).  Both
forms of L<variant> are evaluated for every pair; only the accumulated
statistics leave the GPU.  Prints one JSON line.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def make_pairs(n, seed, dev):
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    x = torch.empty((n, 4), dtype=torch.float64, device=dev).uniform_(-4, 4, generator=g)
    y = torch.empty((n, 4), dtype=torch.float64, device=dev).uniform_(-4, 4, generator=g)
    u = torch.rand(n, dtype=torch.float64, device=dev, generator=g)
    scale = torch.pow(10.0, -4.0 + 2.0 * torch.rand(n, dtype=torch.float64, device=dev,
                                                        generator=g))
    sx = u < 0.005
    sy = (u >= 0.005) & (u < 0.01)
    # scale the small side to |.| = scale along its own direction
    x[sx] = x[sx] / torch.linalg.vector_norm(x[sx], dim=1, keepdim=True) * scale[sx, None]
    y[sy] = y[sy] / torch.linalg.vector_norm(y[sy], dim=1, keepdim=True) * scale[sy, None]
    return x.contiguous(), y.contiguous()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--pairs", type=float, default=1e8)
    p.add_argument("--variant", type=int, default=3)
    p.add_argument("--seed", type=int, default=4)
    p.add_argument("--floor", type=float, default=1e-300)
    a = p.parse_args()
    sys.path.insert(0, ROOT)
    import torch

    import kqed_gb300 as K
    n = int(a.pairs)
    t = K.KernelTemps()
    from benchmarks.clocks import ClockSampler
    x, y = make_pairs(n, a.seed, "cuda")
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    t0 = time.perf_counter()
    st = K.precision_stats(t, a.variant, x.data_ptr(), y.data_ptr(), n, a.floor)
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    cm, cr = st["comp_max"], st["comp_rms"]
    out = {"workload": "L%d, %d pairs, x,y ~ U[-4,4]^4, 1%% with |x| or |y| in [1e-4,1e-2)"
                       % (a.variant, n),
           "metric": "per pair r_c = |L_c(mixed) - L_c(fp64)| / max_c |L_c(fp64)|",
           "pairs_counted": st["pairs"], "pair_max": st["pair_max"], "pair_mean": st["pair_mean"],
           "component_max": {"max": float(cm.max()), "median": float(np.median(cm)),
                             "argmax": int(np.argmax(cm))},
           "component_rms": {"max": float(cr.max()), "median": float(np.median(cr))},
           "seconds": wall, "pairs_per_s_both_forms": n / wall, "clocks": clocks}
    print(json.dumps(out))
    t.free()


if __name__ == "__main__":
    main()
