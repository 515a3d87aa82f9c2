"""Measurement tooling beside bench.py: the workload scripts behind the
summaries under profiles/, the clock sampler, and the FP64 work model of the
roofline.  Not part of the library binding (kqed_gb300)."""
