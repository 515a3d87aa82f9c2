"""The network oracle (oracle/mlp_oracle.py) pinned by finite differences:
its analytic gradient of the mean-square loss (float64, no bf16 rounding)
against central differences on randomly chosen parameters of every block.
Tolerance 1e-6 relative to the gradient's scale."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import mlp_oracle as MO  # noqa: E402


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = MO.init_params(7).astype(np.float64)
    feat = rng.uniform(-1, 1, (16, 3))
    target = rng.normal(size=(16, 39))
    _, g, _ = MO.loss_and_grad(p, feat, target, bf=False)
    for name, (a, b) in MO.BLOCKS.items():
        idx = rng.integers(a, b, 6)
        scale = np.abs(g[a:b]).max()
        for i in idx:
            h = 1e-6 * max(1.0, abs(p[i]))
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            lp, _, _ = MO.loss_and_grad(pp, feat, target, bf=False)
            lm, _, _ = MO.loss_and_grad(pm, feat, target, bf=False)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 * scale + 1e-12, (name, i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    # bf16 keeps 7 fraction bits: one ulp at 1.0 is 2^-7
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9,
                  -2.5e-3])
    r = MO.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie between 1 and 1 + 2^-7: to even
    assert r[2] == 1.0 + 2 ** -6            # tie between 1 + 2^-7 and 1 + 2^-6: to even
    assert r[3] == 1.0                      # below half an ulp
    assert r[4] == 1.0 + 2 ** -7            # above half an ulp
    assert abs(r[5] - v[5]) <= 2 ** -9 * abs(v[5])
