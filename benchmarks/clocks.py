"""GPU clocks and throttle reasons sampled during a timed region.

    clk = ClockSampler(device_index); clk.start(); ... timed work ...; info = clk.stop()

`info` = {"sm_mhz": median SM clock of the samples, "sm_max_mhz": ..., "reasons":
[active throttle reasons among hw_slowdown, hw_thermal_slowdown,
sw_thermal_slowdown, sw_power_cap], "samples": n}.  nvidia-smi is only read
(query mode); no GPU setting is touched.
"""
import subprocess
import threading

import numpy as np

QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]


def summarize(lines):
    """The summary of nvidia-smi CSV lines (no header, no units) in QUERY's
    column order; lines that do not parse are skipped."""
    sm, smax, reasons = [], None, set()
    for ln in lines:
        f = [v.strip() for v in ln.split(",")]
        if len(f) < 8:
            continue
        try:
            sm.append(float(f[1]))
            smax = float(f[2])
        except ValueError:
            continue
        for nm, v in zip(REASONS, f[4:8]):
            if v.lower() == "active":
                reasons.add(nm)
    return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
            "reasons": sorted(reasons), "samples": len(sm)}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.dev)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        return summarize(self.lines)
