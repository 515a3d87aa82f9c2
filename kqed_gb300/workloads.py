"""Seeded synthetic inputs with the shapes of the benchmark configurations.

No public dataset is involved: the (x, y) pairs, lattices and the hadronic
function Pi(x, y) are all synthetic, generated from fixed seeds.
"""
import numpy as np


def config1_pairs(seed=1, n_generic=4096, n_small=64):
    """4096 pairs with components uniform in [-2, 2], plus 64 pairs where one
    side is tiny (a uniform [-1,1] direction scaled by a log-uniform length in
    [1e-6, 1e-3]) to reach the small-|x| / small-|y| branches."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2.0, 2.0, (n_generic, 4))
    y = rng.uniform(-2.0, 2.0, (n_generic, 4))
    d = rng.uniform(-1.0, 1.0, (n_small, 4))
    s = 10.0 ** rng.uniform(-6.0, -3.0, n_small)
    small = d * s[:, None]
    other = rng.uniform(-2.0, 2.0, (n_small, 4))
    h = n_small // 2
    xs = np.vstack([x, small[:h], other[h:]])
    ys = np.vstack([y, other[:h], small[h:]])
    return xs, ys


def lattice_sites(L, a):
    """Sites of a periodic L^4 lattice with spacing a, as minimal-image
    4-vectors a*((n + L/2) mod L - L/2), components in [-L/2, L/2-1]*a."""
    n = np.arange(L)
    c = a * ((n + L // 2) % L - L // 2)
    g = np.stack(np.meshgrid(c, c, c, c, indexing="ij"), axis=-1)
    return np.ascontiguousarray(g.reshape(-1, 4))


def diagonal_x(nx, a):
    """x_k = a*k*(1,1,1,1), k = 0..nx-1."""
    k = np.arange(nx, dtype=np.float64)
    return np.ascontiguousarray(np.outer(k * a, np.ones(4)))


def pi_envelope(x, y):
    """exp(-|y|/2) exp(-|x-y|/2) for every (x_k, y_n): [nx][ny]."""
    ny = np.linalg.norm(y, axis=1)
    nxy = np.linalg.norm(x[:, None, :] - y[None, :, :], axis=2)
    return np.exp(-0.5 * ny)[None, :] * np.exp(-0.5 * nxy)


def pi_synth_numpy(x, y, seed=2):
    """Pi[k][n][c] = N(0,1) * exp(-|y|/2) * exp(-|x-y|/2) (small sizes)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((len(x), len(y), 384))
    return g * pi_envelope(x, y)[:, :, None]


def pi_synth_torch(x, y, seed=2, device="cuda", chunk=4):
    """Same distribution generated on the device with torch (large sizes);
    returns a contiguous float64 tensor [nx][ny][384]."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    xt = torch.as_tensor(x, dtype=torch.float64, device=device)
    yt = torch.as_tensor(y, dtype=torch.float64, device=device)
    out = torch.empty((len(x), len(y), 384), dtype=torch.float64, device=device)
    ny = torch.linalg.vector_norm(yt, dim=1)
    for k0 in range(0, len(x), chunk):
        k1 = min(len(x), k0 + chunk)
        env = torch.exp(-0.5 * ny)[None, :] * torch.exp(
            -0.5 * torch.linalg.vector_norm(xt[k0:k1, None, :] - yt[None, :, :], dim=2))
        blk = torch.randn((k1 - k0, len(y), 384), dtype=torch.float64, device=device,
                          generator=gen)
        blk.mul_(env[:, :, None])
        out[k0:k1].copy_(blk)
        del blk
    return out
