"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

DM trials shard across ranks with no data-path collective: each rank takes an
interleaved share of a 512*N-trial grid (equal work per rank, weak scaling), the
timing is the maximum over ranks, and the folded profiles are gathered on the host
afterwards.  Only one GPU exists in this run, so this
is the coverage of the N > 1 path.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, local = bench.dist_setup()
    wl = bench.WORKLOADS["many_dm_512"]
    grid = bench.dm_grid(wl, r, w)
    t = bench.reduce_max(float(10 + rank), w)
    s = bench.reduce_sum(float(len(grid)), w)
    # the host gather of the per-rank [D][K] profiles puts row i of the grid at i
    prof = np.stack([np.full(4, float(d)) for d in grid])
    full = bench.gather_profiles(prof, w)
    bench.barrier(w)
    q.put((r, grid.tolist(), t, s, full[:, 0].tolist()))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_dm_sharding_and_reductions():
    world = 2
    port = 29000 + (os.getpid() % 2000)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    g0, g1 = np.array(out[0][1]), np.array(out[1][1])
    assert len(g0) == len(g1) == 512  # equal per-rank work
    assert not set(g0.tolist()) & set(g1.tolist())  # disjoint shares
    full = np.sort(np.concatenate([g0, g1]))
    assert len(full) == 1024 and full[0] == 0.0 and abs(full[-1] - 200.0) < 1e-4
    assert all(o[2] == 11.0 for o in out)  # max over ranks
    assert all(o[3] == 1024.0 for o in out)  # total trials
    for o in out:  # every rank holds the whole grid's profiles, in grid order
        np.testing.assert_array_equal(np.array(o[4], np.float32), full)


def test_single_rank_grid_is_the_workload():
    sys.path.insert(0, str(ROOT))
    import bench

    g = bench.dm_grid(bench.WORKLOADS["many_dm_512"])
    np.testing.assert_array_equal(g, np.linspace(0, 200, 512).astype(np.float32))
