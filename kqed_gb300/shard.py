"""Multi-GPU sharding of the fused lattice sum: one process per GPU.

The (x, y) pairs are independent, so a lattice sum splits into contiguous
slabs of sites, one per rank.  Every rank evaluates its slab against all x
points on its own GPU (the tables are replicated, each rank loads its own);
the only collective is a gather of the per-x partial sums (nx doubles per
rank), which every rank then adds in rank order with compensated summation,
so the result does not depend on the collective's internal order.

For generated Pi the slab passes its first site's global index, so every
rank sees the Pi of the whole lattice.

    sums = sharded_lattice_sum(t, 2, xs, ys, seed=7)        # under torchrun

With one rank this is the single-GPU entry point.
"""
import numpy as np

TILE = 64


def site_slab(ny, rank, world, align=TILE):
    """[start, stop) of rank's sites: contiguous slabs of whole 64-site tiles,
    sizes differing by at most one tile."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d not in a world of %d" % (rank, world))
    tiles = (ny + align - 1) // align
    lo = rank * tiles // world
    hi = (rank + 1) * tiles // world
    return min(lo * align, ny), min(hi * align, ny)


def combine_rank_order(parts):
    """Compensated (Neumaier) sum over ranks, in rank order: parts [world][nx]."""
    parts = np.asarray(parts, dtype=np.float64)
    s = np.zeros(parts.shape[1])
    c = np.zeros(parts.shape[1])
    for p in parts:
        t = s + p
        big = np.abs(s) >= np.abs(p)
        c += np.where(big, (s - t) + p, (p - t) + s)
        s = t
    return s + c


def _gpu_local_sum(t, variant, xs, ys_slab, y_offset, pi_slab, seed, stream_id, precision):
    import torch

    import kqed_gb300 as K
    dev = torch.device("cuda", torch.cuda.current_device())
    dx = torch.as_tensor(np.ascontiguousarray(xs), dtype=torch.float64, device=dev)
    dy = torch.as_tensor(np.ascontiguousarray(ys_slab), dtype=torch.float64, device=dev)
    out = torch.zeros(len(xs), dtype=torch.float64, device=dev)
    if len(ys_slab):
        if pi_slab is None:
            K.lattice_sum_synth(t, variant, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys_slab),
                                seed, out.data_ptr(), precision, stream_id=stream_id,
                                y_offset=y_offset)
        else:
            pi = torch.as_tensor(pi_slab, dtype=torch.float64, device=dev).contiguous()
            K.lattice_sum_dev(t, variant, dx.data_ptr(), len(xs), dy.data_ptr(), len(ys_slab),
                              pi.data_ptr(), out.data_ptr(), precision)
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


def sharded_lattice_sum(t, variant, xs, ys, pi=None, seed=None, stream_id=0, precision=0,
                        group=None, local_sum=None):
    """sums[k] = sum over all sites y of L<variant>(x_k, y).Pi(x_k, y), the
    sites split across the ranks of `group` (torch.distributed; a single
    process when it is not initialised).  Pi: pi [nx][ny][384] (each rank
    uses its slab) or the generated Pi of `seed`.  `local_sum` replaces the
    per-rank GPU evaluation (same signature as the default)."""
    import torch.distributed as dist
    if (pi is None) == (seed is None):
        raise ValueError("give exactly one of pi and seed")
    world = dist.get_world_size(group) if dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank(group) if world > 1 else 0
    lo, hi = site_slab(len(ys), rank, world)
    f = local_sum or _gpu_local_sum
    part = f(t, variant, xs, ys[lo:hi], lo, None if pi is None else pi[:, lo:hi], seed,
             stream_id, precision)
    if world == 1:
        return np.asarray(part, dtype=np.float64)
    import torch
    be = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if be == "nccl" else torch.device("cpu")
    mine = torch.as_tensor(np.asarray(part, dtype=np.float64), device=dev)
    gathered = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(gathered, mine, group=group)
    return combine_rank_order([g.cpu().numpy() for g in gathered])
