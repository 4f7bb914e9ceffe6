"""Host logic of the multi-GPU bench path on two CPU ranks (gloo): every rank
takes its own wavelengths of each step (the ranks' sets are disjoint, and the
steps walk the workload's grid: 60 points for the 4000-face sphere, 32 for the
24 000-face dimer), and the timings are reduced to their maximum over ranks
with no other collective."""
import argparse
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


def _rank(rank, world, port, workload, batch, steps, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a = argparse.Namespace(workload=workload)
        mine = np.concatenate([bench.step_wavelengths(a, s, rank, world, batch) for s in range(steps)])
        got = [None] * world
        dist.all_gather_object(got, mine.tolist())
        ms = bench.max_over_ranks(dist, [10.0 + rank, 5.0 - rank], "cpu", torch)
        out.put((rank, got, ms))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("workload,batch,steps", [("sphere4000", 10, 3), ("dimer24k", 4, 4)])
def test_two_ranks_share_the_grid_and_reduce_max(workload, batch, steps):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, workload, batch, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    grid = bench.grid(argparse.Namespace(workload=workload))
    for rank, got, ms in res:
        assert ms == [10.0 + world - 1, 5.0]
        a, b = np.array(got[0]), np.array(got[1])
        assert a.size == b.size == batch * steps
        # one step: the ranks' wavelengths are disjoint grid points
        for s in range(steps):
            sa, sb = a[s * batch:(s + 1) * batch], b[s * batch:(s + 1) * batch]
            assert not set(sa.tolist()) & set(sb.tolist())
        # the steps of two ranks cover the grid once
        assert np.array_equal(np.sort(np.concatenate([a, b])), np.sort(grid))


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, [1.5, 2], "cpu", None) == [1.5, 2.0]
