#!/usr/bin/env python3
"""Benchmark: (x,y) kernel evaluations/s of the fused lattice integrand.

Workload (one step): periodic 24^4 lattice, spacing 0.1, 32 points x_k along
the (1,1,1,1) diagonal, y over all 331,776 sites, kernel L2, synthetic
Pi(x,y) = N(0,1) exp(-|y|/2) exp(-|x-y|/2) of 384 float64 components, and
the fused sum_y sum_c L2_c(x,y) Pi_c(x,y) per x.  One evaluation = one (x,y)
term.  Pi is 32.6 GB per step, far larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` times the device entry point with
inputs resident in HBM, in the precision form given by --precision (fp64:
the plain FP64 form, bit-for-bit the reference's algorithm; fp32: the mixed
form).  Both forms are always timed on the same inputs and reported under
`forms`, with the mixed form's integrand error against the FP64 sums of the
same run.  `e2e` times the host entry point with Pi in page-locked host
memory from the library's allocator: every step the kernels read it there,
over the host link (`pi_route`; KQED_HOST_PI=copy stages it through device
buffers instead).  --impl reference times the reference's CPU
implementation of the same computation on the host cores (the reference
library compiled from its sources when it is available here, else the CPU
restatement under oracle/).
"""
import argparse
import ctypes
import json
import math
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from benchmarks.clocks import ClockSampler  # noqa: E402

METRIC = ("(x,y) kernel evals/s on 1 GB300: plain FP64 vs FP32/surrogate at "
          "≤1e-6 rel err")
UNIT = "evals/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    p.add_argument("--L", type=int, default=24)
    p.add_argument("--spacing", type=float, default=0.1)
    p.add_argument("--nx", type=int, default=32)
    p.add_argument("--variant", type=int, default=2)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--strong", action="store_true",
                   help="N > 1: one lattice, its sites split across the ranks "
                        "(kqed_gb300/shard.py), per-x partial sums gathered and combined")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def x_direction(rank):
    """Weak scaling: rank r evaluates the same number of x points along its own
    diagonal (sign pattern of r), so every rank carries identical work."""
    s = [1.0, 1.0, 1.0, 1.0]
    for b in range(4):
        if (rank >> b) & 1:
            s[3 - b] = -1.0
    return np.array(s)


def cpu_impl():
    """(ctypes lib, kind): the reference library built from its sources when
    present (x86 only), else the CPU restatement."""
    ref = os.path.join(ROOT, "oracle", "_ref", "libkqedref_avx.so")
    if os.path.exists(ref):
        try:
            os.environ["KQEDREF_PATH"] = os.path.join(ROOT, "kqed_gb300")
            L = ctypes.CDLL(ref)
            if L.ref_init_threads(os.cpu_count() or 1) == 0:
                def contract(v, x, y, pi, nt):
                    dp = ctypes.POINTER(ctypes.c_double)
                    d = np.zeros(len(x))
                    L.ref_contract(v, len(x), x.ctypes.data_as(dp), y.ctypes.data_as(dp),
                                   pi.ctypes.data_as(dp), d.ctypes.data_as(dp), nt)
                    return d
                return contract, "reference"
        except OSError:
            pass
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _helpers import oracle_contract

    def contract(v, x, y, pi, nt):
        return oracle_contract(v, x, y, pi, nt)
    return contract, "port"


def cpu_sample(args, xs, ys, pi_host_fn, steps=1):
    """Time the CPU implementation on a bounded sample of the workload: a few
    x points against all sites.  Returns (evals/s, cores, kind, sample,
    checked), checked = {k: (sum_y L.Pi, sum_y |L.Pi|)} of the sampled x
    points, the CPU's lattice sums for the parity check of the GPU's."""
    contract, kind = cpu_impl()
    cores = os.cpu_count() or 1
    ks = [len(xs) // 4, len(xs) // 2, (3 * len(xs)) // 4] if len(xs) >= 4 else [0]
    best = None
    checked = {}
    for _ in range(steps):
        t_tot, n_tot = 0.0, 0
        for k in ks:
            pik = pi_host_fn(k)
            X = np.ascontiguousarray(np.repeat(xs[k:k + 1], len(ys), 0))
            t0 = time.perf_counter()
            d = contract(args.variant, X, ys, pik, cores)
            t_tot += time.perf_counter() - t0
            n_tot += len(ys)
            checked[k] = (math.fsum(d), math.fsum(np.abs(d)))
        rate = n_tot / t_tot
        best = rate if best is None else max(best, rate)
    sample = "%d x points (k=%s) x %d sites, L%d contraction, %d threads" % (
        len(ks), ",".join(str(k) for k in ks), len(ys), args.variant, cores)
    return best, cores, kind, sample, checked


PARITY_TOL = 1e-12


def parity_of(gpu_sums, checked):
    """The GPU's FP64 lattice sums against the CPU implementation's on the
    sampled x points: |S_gpu - S_cpu| / sum_y |L.Pi| (the sum's condition
    scale; the tests use the same bound)."""
    if not checked:
        return None
    rel = {k: abs(float(gpu_sums[k]) - s) / max(a, 1e-300) for k, (s, a) in checked.items()}
    worst = max(rel.values())
    return {"max_rel": worst, "tol": PARITY_TOL, "ok": bool(worst <= PARITY_TOL),
            "x_checked": sorted(int(k) for k in checked),
            "definition": "|S_gpu - S_cpu| / sum_y |L.Pi| per checked x, FP64 form"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from kqed_gb300 import build as B
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_envelope
    os.makedirs(B.OUT, exist_ok=True)
    B.ensure_table(B.build_synth())
    xs = diagonal_x(args.nx, args.spacing)
    ys = lattice_sites(args.L, args.spacing)

    def pi_host(k):
        rng = np.random.default_rng(1000 + k)
        env = pi_envelope(xs[k:k + 1], ys)[0]
        return rng.standard_normal((len(ys), 384)) * env[:, None]

    cache = {}

    def pi_cached(k):
        if k not in cache:
            cache[k] = pi_host(k)
        return cache[k]

    for _ in range(args.warmup):
        cpu_sample(args, xs, ys, pi_cached, steps=1)
    rates = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, cores, kind, sample, _ = cpu_sample(args, xs, ys, pi_cached, steps=1)
        rates.append(r)
    wall = time.perf_counter() - t0
    value = float(np.median(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(args, len(ys)),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def roofline_line(pipes, fp64_equiv, peak64_gflops):
    """The roofline fields: the busier pipe's rate against its probe peak
    (frac <= 1 unless a pipe really runs at its probe rate), each pipe's
    figures, and the FP64-equivalent rate of earlier measurements, labelled
    as such (the algorithm's FP64 operations, now largely executed in
    double-float on the FP32 pipe)."""
    eq = {"achieved": fp64_equiv, "peak": peak64_gflops / 1e3, "unit": "TFLOP/s",
          "frac": fp64_equiv / (peak64_gflops / 1e3),
          "definition": "the algorithm's FP64 operations per pair, counted on its all-FP64 "
                        "evaluation, over the launch time: a value above 1 says the "
                        "double-float stages beat DFMA, not that a pipe is saturated"}
    if not pipes:
        return {"bound": "fp64", "achieved": fp64_equiv, "peak": peak64_gflops / 1e3,
                "unit": "TFLOP/s", "frac": eq["frac"], "fp64_equivalent": eq}
    busier = max(pipes, key=lambda k: pipes[k]["frac"])
    b = pipes[busier]
    return {"bound": "%s pipe (the busier of FP64 and FP32)" % busier, "achieved": b["achieved"],
            "peak": b["peak"], "unit": "TFLOP/s", "frac": b["frac"], "pipes": pipes,
            "fp64_equivalent": eq}


def workload_config(args, ny):
    return {"workload": "fused lattice integrand: kernel L%d, periodic %d^4 lattice, spacing %g, "
                        "%d x points on the diagonal, sum over all sites of L.Pi"
                        % (args.variant, args.L, args.spacing, args.nx),
            "lattice_L": args.L, "spacing": args.spacing, "nx": args.nx, "ny": ny,
            "variant": "L%d" % args.variant, "precision": args.precision,
            "l2": "inputs larger than L2 (Pi is %.1f GB per step)" % (args.nx * ny * 384 * 8 / 1e9)}


def run_gb300(args):
    import torch

    import kqed_gb300 as K
    from benchmarks import flops as F
    from kqed_gb300.workloads import diagonal_x, lattice_sites, pi_synth_torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    t = K.KernelTemps()
    g = t.grid()
    prec = {"fp64": K.KQED_FP64, "fp32": K.KQED_FP32_MIXED}[args.precision]

    if args.strong:
        # strong scaling: every rank takes the same x points and its own slab
        # of the lattice's sites; Pi is the library's generated Pi at the
        # sites' global indices, so the combined sums do not depend on N
        from kqed_gb300.shard import site_slab
        xs = diagonal_x(args.nx, args.spacing)
        ys_all = lattice_sites(args.L, args.spacing)
        lo, hi = site_slab(len(ys_all), rank, world)
        ys = ys_all[lo:hi]
    else:
        xs = diagonal_x(args.nx, args.spacing) * x_direction(rank)[None, :]
        ys = lattice_sites(args.L, args.spacing)
    nx, ny = len(xs), len(ys)
    dx = torch.as_tensor(xs, dtype=torch.float64, device=dev)
    dy = torch.as_tensor(ys, dtype=torch.float64, device=dev)
    if args.strong:
        pi = torch.empty((nx, ny, 384), dtype=torch.float64, device=dev)
        K.pi_synth_dev(dx.data_ptr(), nx, dy.data_ptr(), ny, 7, pi.data_ptr(), y_offset=lo)
        torch.cuda.synchronize(dev)
    else:
        pi = pi_synth_torch(xs, ys, seed=2 + rank, device=dev)
    sums = torch.empty(nx, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(p=None):
        K.lattice_sum_dev(t, args.variant, dx.data_ptr(), nx, dy.data_ptr(), ny, pi.data_ptr(),
                          sums.data_ptr(), prec if p is None else p, stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)

    # ---- device-resident timing
    clocks = ClockSampler(dev.index if dev.index is not None else 0)
    barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    time.sleep(0.3)
    K.profile(True)
    l0 = K.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    clk = clocks.stop()
    launches = K.launch_count() - l0
    ms_total = e0.elapsed_time(e1)
    kern_ms, kern_n = K.profile_read()
    K.profile(False)
    ms_step = ms_total / args.steps
    if world > 1:
        mt = torch.tensor([ms_step], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(mt, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(mt.item())
    # weak: every rank its own lattice; strong: the ranks' slabs make one lattice
    total_pairs = nx * len(ys_all) if args.strong else world * nx * ny
    value = total_pairs / (ms_step / 1e3)

    # ---- both precision forms on the same resident inputs: time and the
    #      mixed form's integrand error against the FP64 sums
    forms = {}
    fsums = {}
    for name, pm in (("fp64", K.KQED_FP64), ("fp32_mixed", K.KQED_FP32_MIXED)):
        for _ in range(2):
            step(pm)
        torch.cuda.synchronize(dev)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            step(pm)
        f1.record(stream)
        torch.cuda.synchronize(dev)
        fms = f0.elapsed_time(f1) / args.steps
        fsums[name] = sums.cpu().numpy().copy()
        forms[name] = {"value": total_pairs / (fms / 1e3), "ms_per_step": fms}
    ref = fsums["fp64"]
    err = np.abs(fsums["fp32_mixed"] - ref)
    rms = float(np.sqrt(np.mean(ref ** 2)))
    live = np.abs(ref) > 1e-12 * max(rms, 1e-300)
    forms["fp32_mixed"].update({
        "speedup_vs_fp64": forms["fp64"]["ms_per_step"] / forms["fp32_mixed"]["ms_per_step"],
        "err_vs_fp64": {
            "definition": "per x: |S_fp32 - S_fp64| / rms_x(S_fp64), S = sum_y L.Pi",
            "max": float(err.max() / rms) if rms > 0 else None,
            "median": float(np.median(err) / rms) if rms > 0 else None,
            "max_rel_own": float((err[live] / np.abs(ref[live])).max()) if live.any() else None}})

    # ---- roofline of the dominant kernels (record + assembly, FP64 form):
    #      the operations each pipe executes per launch (calibrated per
    #      kernel and pipe from ncu's executed-instruction counters) over the
    #      event-timed duration, against the library's FMA-chain probes of
    #      the FP64 and FP32 pipes; the busier pipe sets the bound
    peak_gflops = K.fp64_peak_gflops()
    peak32_gflops = K.fp32_peak_gflops()
    flops_launch = F.lattice_flops(xs, ys, g["XX"], g["nfx"], args.variant)
    kavg_ms = kern_ms / max(kern_n, 1)
    achieved = flops_launch / (kavg_ms / 1e3) / 1e12
    pipes = {}
    for pipe, peak in (("fp64", peak_gflops), ("fp32", peak32_gflops)):
        parts = [F.lattice_flops(xs, ys, g["XX"], g["nfx"], args.variant, model="%s_%s" % (k, pipe))
                 for k in ("record", "assembly")]
        if any(p is None for p in parts):
            continue
        fl = float(sum(parts))
        a_t = fl / (kavg_ms / 1e3) / 1e12
        pipes[pipe] = {"flops_per_launch": fl, "achieved": a_t, "peak": peak / 1e3,
                       "frac": a_t / (peak / 1e3), "record_share_of_flops": parts[0] / fl}

    # ---- end to end through the host entry point (Pi from pinned memory)
    def measure_e2e(pi):
        # the caller's Pi in page-locked, device-mapped memory from the
        # library's allocator, which the kernels read in place
        pinned = K.PinnedArray(tuple(pi.shape))
        pi_host = torch.from_numpy(pinned.array)
        pi_host.copy_(pi)
        xh = np.ascontiguousarray(xs)
        yh = np.ascontiguousarray(ys)
        sh = np.zeros(nx)
        dp = ctypes.POINTER(ctypes.c_double)
        lib = K.lib()

        def e2e_step():
            rc = lib.kqed_lattice_sum(t.ptr, args.variant, nx, xh.ctypes.data_as(dp), ny,
                                      yh.ctypes.data_as(dp),
                                      ctypes.cast(pi_host.data_ptr(), dp), sh.ctypes.data_as(dp), prec)
            if rc != 0:
                raise RuntimeError(lib.kqed_last_error().decode())

        e2e_step()
        barrier()
        K.profile(True)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        barrier()
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        e2e_kern_ms, _ = K.profile_read()
        e2e_copy_ms, _ = K.profile_read_copies()
        K.profile(False)
        if world > 1:
            mt = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
            torch.distributed.all_reduce(mt, op=torch.distributed.ReduceOp.MAX)
            e2e_s = float(mt.item())
        # host->device copy rate right after (the same pinned buffer, 1 GB
        # pieces): the bound of the staged route, which the in-place route,
        # reading Pi with the GPU's own loads, can pass
        scratch = torch.empty(min(pi_host.numel(), 1 << 27), dtype=torch.float64, device=dev)
        flat = pi_host.view(-1)
        torch.cuda.synchronize(dev)
        c0 = time.perf_counter()
        moved = 0
        for o in range(0, flat.numel(), scratch.numel()):
            n = min(scratch.numel(), flat.numel() - o)
            scratch[:n].copy_(flat[o:o + n], non_blocking=True)
            moved += n * 8
        torch.cuda.synchronize(dev)
        h2d_gbs = moved / (time.perf_counter() - c0) / 1e9
        del scratch
        in_place = (K.pinned_contains(pi_host.data_ptr(), pi_host.numel() * 8)
                    and os.environ.get("KQED_HOST_PI") != "copy")
        e2e = {"value": total_pairs / e2e_s, "unit": UNIT,
               "pi_route": ("read in place by the kernels over the host link" if in_place
                            else "staged through device buffers by copies"),
               "h2d_bytes_per_step": int(pi_host.numel() * 8 + xh.nbytes + yh.nbytes),
               "d2h_bytes_per_step": int(sh.nbytes),
               "precision": args.precision,
               "h2d_link_gbs_measured": h2d_gbs,
               "ms_per_step": e2e_s * 1e3,
               # summed over the lattice launches of both streams, which overlap
               "kernel_ms_per_step": e2e_kern_ms / args.e2e_steps,
               "copy_ms_per_step": e2e_copy_ms / args.e2e_steps,
               "h2d_gbs_during_step": pi_host.numel() * 8 / (e2e_copy_ms / args.e2e_steps / 1e3) / 1e9
               if e2e_copy_ms > 0 else None,
               "h2d_gbs_effective": pi_host.numel() * 8 / e2e_s / 1e9,
               "copy_bound_evals_per_s": total_pairs / (pi_host.numel() * 8 / (h2d_gbs * 1e9))}
        return e2e, pi_host, pinned

    pinned = None
    if args.e2e_steps > 0:
        e2e, pi_host, pinned = measure_e2e(pi)
        del pi
        torch.cuda.empty_cache()
    else:
        e2e, pi_host = None, pi.cpu()
        del pi

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        def pi_k(k):
            return pi_host[k].numpy()
        r, cores, kind, sample, checked = cpu_sample(args, xs, ys, pi_k, steps=1)
        cpu = {"value": r, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample}
        parity = parity_of(fsums["fp64"], checked)
        parity["against"] = kind

    # strong scaling: the per-x partial sums of the slabs, gathered and
    # added in rank order (the only collective: nx doubles per rank)
    if args.strong and world > 1:
        from kqed_gb300.shard import combine_rank_order
        mine = torch.as_tensor(fsums["fp64"], device=dev)
        got = [torch.empty_like(mine) for _ in range(world)]
        torch.distributed.all_gather(got, mine)
        fsums["fp64"] = combine_rank_order([g.cpu().numpy() for g in got])

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "strong" if args.strong else "weak",
            "vs_baseline": None,
            "dtype": {"fp64": "f64 (double-float assembly)", "fp32": "f32+f64"}[args.precision],
            "data": "synthetic",
            "config": workload_config(args, len(ys_all) if args.strong else ny) | (
                {"parallelism": "sites sharded over %d ranks (kqed_gb300/shard.py); Pi "
                                "generated by the library at global site indices (seed 7)" % world}
                if args.strong else {}),
            "e2e": e2e,
            "forms": forms,
            "gpu_launches": launches,
            "roofline": roofline_line(pipes, achieved, peak_gflops) | {
                         "traffic": (F.table().get("TRAFFIC_BYTES_PER_PAIR", 0) * nx * ny
                                     if args.precision == "fp64" else None),
                         "traffic_unit": "bytes per launch (record + assembly kernels)",
                         "traffic_source": F.table().get("traffic_source"),
                         "kernel": "lattice_rec_kernel<double> + lattice_asm_kernel<double>"
                                   if args.precision == "fp64" else
                                   "lattice_rec_lean_kernel + lattice_rec_kernel<float> + "
                                   "lattice_asm_kernel<float>",
                         "kernel_ms": kavg_ms,
                         "flops_per_launch": flops_launch,
                         "flops_source": F.table().get("source"),
                         "peak_source": "FP64 and FP32 FMA-chain probes run by this bench "
                                        "(MEASURED_PEAKS.json has neither)"},
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clk,
            "checksum": [float(v) for v in fsums["fp64"][:4]],
        }
        print(json.dumps(line), flush=True)
    pi_host = None
    if pinned is not None:
        pinned.free()
    t.free()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
