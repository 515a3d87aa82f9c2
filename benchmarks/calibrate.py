"""Calibration of the work model in flops.py: the FP64 and the FP32 operations
the lattice kernels execute per pair, per kernel.

  python -m benchmarks.calibrate --run            launches one fused lattice sum (L2)
                                                  per branch-uniform case (a record kernel
                                                  and an assembly kernel each); run it
                                                  under ncu with the FP64 and FP32
                                                  instruction counters
  python -m benchmarks.calibrate --fit CSV        fits, per kernel and pipe, PER_K /
                                                  FIXED / AXIS from the ncu CSV and writes
                                                  flops_table.json

Cases: one x point against 4096 sites of a shifted 8^4 lattice (no site is 0
or equal to x), at |x| in several grid cells (different Chebyshev lengths),
plus x = 0 (every pair takes the x = 0 form).  Per-pair flops of a pipe are
the executed FMA x 2 + ADD + MUL thread instructions of that precision
(DFMA/DADD/DMUL, FFMA/FADD/FMUL) of the case's record or assembly kernel
divided by its pairs.
"""
import argparse
import csv
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CASES = os.path.join(HERE, "_build", "calibration_cases.json")
XMAGS = [0.0, 0.3, 1.0, 2.0, 3.5, 5.0, 6.2]
VARIANT = 2


def sites():
    n = np.arange(8)
    c = 0.3 * (n - 3.5)
    g = np.stack(np.meshgrid(c, c, c, c, indexing="ij"), axis=-1)
    return np.ascontiguousarray(g.reshape(-1, 4))


def run():
    import torch

    sys.path.insert(0, ROOT)
    import kqed_gb300 as K
    t = K.KernelTemps()
    g = t.grid()
    ys = sites()
    dy = torch.as_tensor(ys, device="cuda")
    cases = []
    for m in XMAGS:
        xv = np.array([[0.5, 0.5, 0.5, 0.5]]) * m
        dx = torch.as_tensor(xv, device="cuda")
        pi = torch.randn((1, len(ys), 384), dtype=torch.float64, device="cuda")
        s = torch.zeros(1, dtype=torch.float64, device="cuda")
        K.lattice_sum_dev(t, VARIANT, dx.data_ptr(), 1, dy.data_ptr(), len(ys), pi.data_ptr(),
                          s.data_ptr())
        torch.cuda.synchronize()
        if m == 0.0:
            ktop = 0
        else:
            X = np.sqrt(max(float(xv[0] @ xv[0]), 1e-7))
            ix = max(0, min(int(np.searchsorted(g["XX"], X, side="right") - 1), len(g["XX"]) - 1))
            ix2 = min(ix + 1, len(g["XX"]) - 1)
            ktop = int(max(g["nfx"][ix], g["nfx"][ix2]) + 2)
        cases.append({"xmag": m, "pairs": len(ys), "ktop": ktop})
    os.makedirs(os.path.dirname(CASES), exist_ok=True)
    with open(CASES, "w") as f:
        json.dump(cases, f)
    print(json.dumps(cases))
    t.free()


def fit(path, cases_path):
    cases = json.load(open(cases_path))
    per_launch = {}
    rows = list(csv.reader(open(path)))
    hdr = None
    for r in rows:
        if r and r[0] == "ID":
            hdr = r
            continue
        if not hdr or len(r) != len(hdr):
            continue
        d = dict(zip(hdr, r))
        name = d["Kernel Name"]
        if "lattice_rec_kernel" not in name and "lattice_asm_kernel" not in name:
            continue
        v = float(d["Metric Value"].replace(",", ""))
        per_launch.setdefault(int(d["ID"]), {})[d["Metric Name"]] = v
    ids = sorted(per_launch)
    if len(ids) != 2 * len(cases):
        raise SystemExit("expected %d lattice kernel launches, found %d" % (2 * len(cases), len(ids)))
    ops = {"fp64": ("dfma", "dadd", "dmul"), "fp32": ("ffma", "fadd", "fmul")}

    def count(m, pipe):
        f, a, mu = ops[pipe]
        g = lambda o: m.get("smsp__sass_thread_inst_executed_op_%s_pred_on.sum" % o, 0.0)
        return 2 * g(f) + g(a) + g(mu)

    table = {"source": "ncu executed FMA x 2 + ADD + MUL thread instructions of "
                       "lattice_rec_kernel<double> and lattice_asm_kernel<double> (FP64 form), "
                       "L2, benchmarks/calibrate.py",
             "CONTRACT": 0.0, "CONTRACT_EXTRA": 0.0, "cases": cases, "kernels": {}}
    for kname, off in (("record", 0), ("assembly", 1)):
        for pipe in ("fp64", "fp32"):
            pts, axis = [], None
            for i, c in enumerate(cases):
                fl = count(per_launch[ids[2 * i + off]], pipe) / c["pairs"]
                c["%s_%s" % (kname, pipe)] = fl
                if c["ktop"] == 0:
                    axis = fl
                else:
                    pts.append((c["ktop"], fl))
            kt = np.array([p[0] for p in pts], float)
            fl = np.array([p[1] for p in pts], float)
            A = np.vstack([kt, np.ones_like(kt)]).T
            (per_k, fixed), _, _, _ = np.linalg.lstsq(A, fl, rcond=None)
            table["kernels"]["%s_%s" % (kname, pipe)] = {
                "PER_K": float(per_k), "FIXED": float(fixed), "AXIS": float(axis)}
    # the FP64-equivalent model of earlier versions (all FP64 operations of
    # both kernels, counted when the assembly ran in FP64) is kept as such
    old = {}
    prev = os.path.join(HERE, "flops_table.json")
    if os.path.exists(prev):
        old = json.load(open(prev))
    for k in ("PER_K", "FIXED", "AXIS", "TRAFFIC_BYTES_PER_PAIR", "traffic_source"):
        if k in old:
            table[k] = old[k]
    with open(os.path.join(HERE, "flops_table.json"), "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps(table, indent=1))


if __name__ == "__main__":
    p = argparse.ArgumentParser()
    p.add_argument("--run", action="store_true")
    p.add_argument("--fit")
    p.add_argument("--cases", default=CASES)
    a = p.parse_args()
    if a.run:
        run()
    elif a.fit:
        fit(a.fit, a.cases)
