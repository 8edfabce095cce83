"""The DM-sharded multi-rank path on one GPU (GPU): two gloo ranks, each a separate
process running the engine on its interleaved share of the DM grid (no collective on
the data path; the ranks' kernels never wait on one another), then the host gather of
the [D][K] folded profiles (bench.gather_profiles).  The gathered grid must equal a
single-process run over all trials: same counts, profiles within 1e-6 (the fused
fold's per-CTA float sums may add in another order)."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
W = dict(bw=64e6, centre=1400e6, n_dms=32, dm_lo=0.0, dm_hi=200.0, fftpoint=1 << 18, batch=8, nbins=128,
         samples=1 << 22, period=0.033, inject_dm=123.4, snr_db=-10.0, duty=0.05)


def _fold(rank, world):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "acceleratedms-osm_gb300"))
    import bench
    import pymsosm as eng

    bw, f0 = np.float32(W["bw"]), bench.f0_of(W)
    dms = bench.dm_grid(W, rank, world) if world > 1 else np.linspace(W["dm_lo"], W["dm_hi"], 2 * W["n_dms"]).astype(np.float32)
    x = eng.Simulator(bw, f0, np.float32(W["inject_dm"]), np.float32(W["period"]), kind=eng.SIM_GAUSSIAN,
                      duty=W["duty"], snr_db=W["snr_db"], seed=2).generate(W["samples"])
    m = eng.MsosmGpuBatch(bw, dms, f0).initialize(W["fftpoint"], W["batch"], eng.IN_C64, eng.OUT_NONE)
    n = m.batch * m.M
    fold = eng.FoldGpu(np.float32(W["period"]), bw, n, W["nbins"], len(dms))
    m.attach_fold(fold)
    for s in range(W["samples"] // n):
        m.filter_block(np.ascontiguousarray(x[s * n:(s + 1) * n]))
    m.synchronize()
    folded, _, cnt = fold.read()
    return bench, dms, folded, cnt


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK="0")
    sys.path.insert(0, str(ROOT))
    import bench

    bench.dist_setup()
    _, dms, folded, cnt = _fold(rank, world)
    full = bench.gather_profiles(folded, world)
    full_cnt = bench.gather_profiles(cnt.astype(np.float64), world)
    if rank == 0:
        q.put((full, full_cnt))
    import torch.distributed as dist

    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gather_equals_one_process():
    world = 2
    port = 31000 + (os.getpid() % 2000)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    full, full_cnt = q.get(timeout=600)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    _, dms, one, cnt = _fold(0, 1)
    assert full.shape == one.shape == (2 * W["n_dms"], W["nbins"])
    assert np.array_equal(full_cnt, cnt.astype(np.float64))
    rel = np.abs(full - one).max() / np.abs(one).max()
    assert rel < 1e-6, rel
