"""Calibration of the FP64 work model in flops.py.

  python -m benchmarks.calibrate --run            launches one fused lattice sum (L2)
                                                  per branch-uniform case (a record kernel
                                                  and an assembly kernel each); run it
                                                  under ncu with the FP64 instruction
                                                  counters
  python -m benchmarks.calibrate --fit CSV        fits PER_K / FIXED / AXIS from the ncu CSV
                                                  and writes flops_table.json

Cases: one x point against 4096 sites of a shifted 8^4 lattice (no site is 0
or equal to x), at |x| in several grid cells (different Chebyshev lengths),
plus x = 0 (every pair takes the x = 0 form).  Per-pair FP64 flops are the
executed DFMA x 2 + DADD + DMUL of the case's lattice record and assembly
kernels divided by its pairs.
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
    launches = []
    for i in range(len(cases)):
        a, b = per_launch[ids[2 * i]], per_launch[ids[2 * i + 1]]
        launches.append({m: a.get(m, 0.0) + b.get(m, 0.0) for m in set(a) | set(b)})
    pts = []
    axis = None
    for c, m in zip(cases, launches):
        fl = (2 * m["smsp__sass_thread_inst_executed_op_dfma_pred_on.sum"] +
              m["smsp__sass_thread_inst_executed_op_dadd_pred_on.sum"] +
              m["smsp__sass_thread_inst_executed_op_dmul_pred_on.sum"]) / c["pairs"]
        c["flops_per_pair"] = fl
        rd = m.get("dram__bytes_read.sum")
        if c["ktop"] == 0:
            axis = fl
        else:
            pts.append((c["ktop"], fl))
    kt = np.array([p[0] for p in pts], float)
    fl = np.array([p[1] for p in pts], float)
    A = np.vstack([kt, np.ones_like(kt)]).T
    (per_k, fixed), res, _, _ = np.linalg.lstsq(A, fl, rcond=None)
    table = {"PER_K": float(per_k), "FIXED": float(fixed), "AXIS": float(axis), "CONTRACT": 0.0,
             "CONTRACT_EXTRA": 0.0,
             "source": "ncu executed FP64 ops of lattice_rec_kernel + lattice_asm_kernel "
                       "(FP64 form), L2, benchmarks/calibrate.py",
             "cases": cases}
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
