"""Multi-rank sharding of the fused lattice sum, on CPU: two gloo ranks,
each evaluating its slab of sites with the oracle in place of its GPU; the
gathered, rank-ordered sum equals the single-process oracle sum (relative
1e-13: only the grouping of the compensated additions differs), for stored
and generated Pi, and slabs tile the sites exactly."""
import os
import socket

import numpy as np
import pytest

from _helpers import oracle_contract, oracle_pi_synth


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_local(t, variant, xs, ys_slab, y_offset, pi_slab, seed, stream_id, precision):
    if len(ys_slab) == 0:
        return np.zeros(len(xs))
    if pi_slab is None:
        pi_slab = oracle_pi_synth(xs, ys_slab, seed, stream=stream_id, n0=y_offset)
    X = np.repeat(xs, len(ys_slab), 0)
    Y = np.tile(ys_slab, (len(xs), 1))
    return oracle_contract(variant, X, Y, np.ascontiguousarray(pi_slab).reshape(-1, 384)) \
        .reshape(len(xs), -1).sum(1)


def _inputs():
    from kqed_gb300.workloads import diagonal_x, lattice_sites
    ys = lattice_sites(5, 0.25)                     # 625 sites: ragged last tile
    xs = diagonal_x(3, 0.25) + 0.01
    rng = np.random.default_rng(8)
    pi = rng.standard_normal((len(xs), len(ys), 384))
    return xs, ys, pi


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from kqed_gb300.shard import sharded_lattice_sum
    xs, ys, pi = _inputs()
    out = {}
    for v in (0, 2):
        out[("pi", v)] = sharded_lattice_sum(None, v, xs, ys, pi=pi, local_sum=_oracle_local)
        out[("seed", v)] = sharded_lattice_sum(None, v, xs, ys, seed=21, stream_id=1,
                                               local_sum=_oracle_local)
    dist.destroy_process_group()
    q.put((rank, out))


def test_site_slabs_tile_the_lattice():
    from kqed_gb300.shard import site_slab
    for ny in (1, 63, 64, 625, 331776):
        for world in (1, 2, 3, 8):
            cover = []
            for r in range(world):
                lo, hi = site_slab(ny, r, world)
                assert lo % 64 == 0 and lo <= hi
                cover.extend(range(lo, hi))
            assert cover == list(range(ny))
    with pytest.raises(ValueError):
        site_slab(10, 2, 2)


def test_two_gloo_ranks_reproduce_the_single_process_sum():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    xs, ys, pi = _inputs()
    for v in (0, 2):
        full = _oracle_local(None, v, xs, ys, 0, pi, None, 0, 0)
        fullg = _oracle_local(None, v, xs, ys, 0, None, 21, 1, 0)
        for r in (0, 1):
            np.testing.assert_allclose(res[r][("pi", v)], full, rtol=1e-13,
                                       atol=1e-13 * np.abs(full).max())
            np.testing.assert_allclose(res[r][("seed", v)], fullg, rtol=1e-13,
                                       atol=1e-13 * np.abs(fullg).max())
        assert np.array_equal(res[0][("pi", v)], res[1][("pi", v)])


def test_c_abi_shard_helpers_match_the_python_design():
    """kqed_shard_slab / kqed_shard_combine (the C callers' form of the
    sharding) give shard.py's slabs and its rank-order compensated sums, bit
    for bit; host code only"""
    import ctypes

    from kqed_gb300 import build as B
    B.build()
    import kqed_gb300 as K
    from kqed_gb300.shard import combine_rank_order, site_slab
    L = K.lib()
    L.kqed_shard_slab.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    L.kqed_shard_combine.argtypes = [ctypes.c_size_t, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]
    b, e = ctypes.c_size_t(), ctypes.c_size_t()
    for ny in (0, 1, 63, 64, 65, 1000, 331776, 5308416):
        for world in (1, 2, 3, 4, 7, 8):
            for rank in range(world):
                assert L.kqed_shard_slab(ny, rank, world, ctypes.byref(b), ctypes.byref(e)) == 0
                assert (b.value, e.value) == site_slab(ny, rank, world)
    assert L.kqed_shard_slab(10, 2, 2, ctypes.byref(b), ctypes.byref(e)) != 0
    rng = np.random.default_rng(9)
    dp = ctypes.POINTER(ctypes.c_double)
    for world in (1, 2, 5, 8):
        parts = rng.standard_normal((world, 32)) * 10.0 ** rng.integers(-8, 8, (world, 32))
        parts = np.ascontiguousarray(parts)
        out = np.zeros(32)
        assert L.kqed_shard_combine(32, world, parts.ctypes.data_as(dp), out.ctypes.data_as(dp)) == 0
        assert np.array_equal(out, combine_rank_order(parts))
