"""Composite kernels on one GPU: the reference's own timed loop and a
batch of lattice pairs, against the CPU.

  python -m benchmarks.composite_workload [--which 5] [--n 65536] [--steps 5]

--which numbers the composite as enum kqed_composite (5 =
compute_con_kernelsM_L2, the reference's timed call).  Two workloads:
1. "stress": the reference's stress test (src/amu_forlattice.c:1402-1432):
   8192 calls of compute_con_kernelsM_L2 at x = (1,2,3,4), y = (1,1,1,1),
   M = (0, 0.5, 1, 1.5) -- here one batch of those 8192 identical pairs;
2. "lattice": --n pairs of sites of a periodic 24^4 lattice at spacing 0.1
   (seeded, x and y drawn independently, x = y and x = 0 included when
   drawn), M as above.
For each: FP64 and mixed forms with device-resident inputs and outputs
(CUDA events, after warm-up; clocks sampled), and e2e through the host
entry point kqed_composite_batch with pinned host buffers (inputs copied
in, the output structs copied out inside the timed region).  CPU: the
reference library (x86 build here) or the oracle port, all host cores, on
a bounded sample of the lattice pairs.  Parity: the GPU's FP64 output
against the CPU's on that sample, max |d| / scale, scale = the largest |L0|
the composite combines.  Prints one JSON line.
"""
import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
M4 = np.array([0.0, 0.5, 1.0, 1.5])


def lattice_pairs(n, L=24, a=0.1, seed=17):
    rng = np.random.default_rng(seed)
    h = L // 2
    x = a * (rng.integers(0, L, (n, 4)) - h).astype(np.float64)
    y = a * (rng.integers(0, L, (n, 4)) - h).astype(np.float64)
    return x, y


def cpu_impl(which, M):
    """(fn(x, y, nthreads) -> out, kind): the reference library's composite
    when built here, else the oracle's restatement"""
    dp = ctypes.POINTER(ctypes.c_double)
    ref = os.path.join(ROOT, "oracle", "_ref", "libkqedref_avx.so")
    if os.path.exists(ref):
        os.environ["KQEDREF_PATH"] = os.path.join(ROOT, "kqed_gb300")
        L = ctypes.CDLL(ref)
        if L.ref_init_threads(os.cpu_count() or 1) == 0:
            L.ref_composite_size.restype = ctypes.c_long

            def run(x, y, nt):
                out = np.zeros((len(x), L.ref_composite_size(which)))
                L.ref_composite(which, M.ctypes.data_as(dp), len(x), x.ctypes.data_as(dp),
                                y.ctypes.data_as(dp), out.ctypes.data_as(dp), nt)
                return out
            return run, "reference"
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _helpers import oracle_composite
    return (lambda x, y, nt: oracle_composite(which, x, y, M, nt)), "port"


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--which", type=int, default=5)
    p.add_argument("--n", type=int, default=65536)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--cpu-pairs", type=int, default=2048)
    a = p.parse_args()
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch

    import kqed_gb300 as K
    from _helpers import COMPOSITES, composite_scale
    from benchmarks.clocks import ClockSampler
    M = M4 if a.which != K.KQED_MKERNEL_L2 else M4[2:3]
    t = K.KernelTemps()
    size = K.composite_size(a.which)
    L = K.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    res = {}
    stress = (np.tile([[1.0, 2.0, 3.0, 4.0]], (8192, 1)), np.ones((8192, 4)))
    for wname, (x, y) in (("stress", stress), ("lattice", lattice_pairs(a.n))):
        n = len(x)
        dx = torch.as_tensor(x, device="cuda")
        dy = torch.as_tensor(y, device="cuda")
        out = torch.empty((n, size), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream()
        r = {"pairs": n, "output_bytes_per_pair": size * 8}
        for form, prec in (("fp64", K.KQED_FP64), ("fp32_mixed", K.KQED_FP32_MIXED)):
            def step():
                K.composite_batch_dev(t, a.which, dx.data_ptr(), dy.data_ptr(), out.data_ptr(), n,
                                      M, prec, stream=stream.cuda_stream)
            for _ in range(a.warmup):
                step()
            torch.cuda.synchronize()
            clk = ClockSampler(torch.cuda.current_device())
            clk.start()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(a.steps):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / a.steps
            r[form] = {"ms_per_step": ms, "pairs_per_s": n / (ms / 1e3), "clocks": clk.stop()}
            if form == "fp64":
                got64 = out[: a.cpu_pairs].cpu().numpy()
        r["fp32_mixed"]["speedup_vs_fp64"] = r["fp64"]["ms_per_step"] / r["fp32_mixed"]["ms_per_step"]
        # e2e: host entry point, pinned buffers
        hx = torch.as_tensor(x).pin_memory()
        hy = torch.as_tensor(y).pin_memory()
        ho = torch.empty((n, size), dtype=torch.float64).pin_memory()
        Mv = np.ascontiguousarray(M)
        def e2e():
            rc = L.kqed_composite_batch(t.ptr, a.which, Mv.ctypes.data_as(dp), n,
                                        ctypes.cast(hx.data_ptr(), dp), ctypes.cast(hy.data_ptr(), dp),
                                        ctypes.cast(ho.data_ptr(), dp), K.KQED_FP64)
            assert rc == 0, L.kqed_last_error()
        e2e()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            e2e()
        dt = (time.perf_counter() - t0) / a.steps
        r["e2e_fp64"] = {"ms_per_step": dt * 1e3, "pairs_per_s": n / dt,
                         "h2d_bytes_per_step": 2 * n * 32, "d2h_bytes_per_step": n * size * 8}
        # CPU baseline and parity on a bounded sample
        m = min(a.cpu_pairs, n)
        fn, kind = cpu_impl(a.which, np.ascontiguousarray(M))
        cores = os.cpu_count() or 1
        xs, ys = np.ascontiguousarray(x[:m]), np.ascontiguousarray(y[:m])
        t0 = time.perf_counter()
        ref = fn(xs, ys, cores)
        dt = time.perf_counter() - t0
        r["cpu"] = {"pairs_per_s": m / dt, "kind": kind, "cores": cores,
                    "sample": "first %d pairs" % m}
        scale = composite_scale(a.which, xs, ys)
        d = np.abs(got64[:m] - ref).max(1) / scale
        r["parity"] = {"max_rel_to_scale": float(d.max()), "tol": 1e-12,
                       "ok": bool(d.max() <= 1e-12), "against": kind}
        r["gpu_vs_cpu"] = r["fp64"]["pairs_per_s"] / r["cpu"]["pairs_per_s"]
        res[wname] = r
    print(json.dumps({"composite": COMPOSITES[a.which], "which": a.which, "M": list(M),
                      "workloads": {"stress": "the reference's stress test: 8192 identical "
                                              "pairs x=(1,2,3,4), y=(1,1,1,1)",
                                    "lattice": "%d pairs of sites of a 24^4 lattice, spacing "
                                               "0.1 (seed 17)" % a.n},
                      **res}))
    t.free()


if __name__ == "__main__":
    main()
