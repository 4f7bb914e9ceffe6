"""Host logic of the multi-GPU bench path on two CPU ranks (gloo): every rank
takes its own wavelengths of each step (the ranks' sets are disjoint, and the
steps walk the 60-point grid), and the timings are reduced to their maximum
over ranks with no other collective."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, batch, steps, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = np.concatenate([bench.step_wavelengths(s, rank, world, batch) for s in range(steps)])
        got = [None] * world
        dist.all_gather_object(got, mine.tolist())
        ms = bench.max_over_ranks(dist, [10.0 + rank, 5.0 - rank], "cpu", torch)
        out.put((rank, got, ms))
    finally:
        dist.destroy_process_group()


def test_two_ranks_share_the_grid_and_reduce_max():
    world, batch, steps = 2, 10, 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, batch, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    grid = bench.grid()
    for rank, got, ms in res:
        assert ms == [10.0 + world - 1, 5.0]
        a, b = np.array(got[0]), np.array(got[1])
        assert a.size == b.size == batch * steps
        # one step: the ranks' wavelengths are disjoint grid points
        for s in range(steps):
            sa, sb = a[s * batch:(s + 1) * batch], b[s * batch:(s + 1) * batch]
            assert not set(sa.tolist()) & set(sb.tolist())
        # three steps of two ranks x 10 wavelengths cover the 60-point grid once
        assert np.array_equal(np.sort(np.concatenate([a, b])), np.sort(grid))


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, [1.5, 2], "cpu", None) == [1.5, 2.0]
