"""CUDA-graph capture of a processor's steps (msosm_graph_*) through the C ABI (GPU).

A handle replays a captured graph of one ring period of steps three times over
refilled device input; a second handle runs the same steps with msosm_process.  Both fold every DM and
write the series: the series of the last step must be identical and the folded
profiles equal to the fused fold's float-sum order (counts may differ by a sample at
a bin edge, since the graph advances the fold phase on the device)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 2])
def test_graph_replays_equal_process_calls(eng, precision):
    torch = pytest.importorskip("torch")
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    dms = np.linspace(80.0, 160.0, 24).astype(np.float32)
    F, B, K, period = 1 << 18, 4, 256, np.float32(0.0051)
    mk = lambda: eng.MsosmGpuBatch(bw, dms, f0).initialize(F, B, eng.IN_C64, eng.OUT_C64).set_precision(precision)
    a, g = mk(), mk()
    n = B * a.M
    fa = eng.FoldGpu(period, bw, n, K, len(dms))
    fg = eng.FoldGpu(period, bw, n, K, len(dms))
    a.attach_fold(fa)
    g.attach_fold(fg)
    rp = g.ring_blocks // B
    nsteps = rp * 2 // np.gcd(rp, 2)  # the ring's period in steps (slots and tail buffer)
    sim = eng.Simulator(bw, f0, np.float32(123.4), period, kind=eng.SIM_GAUSSIAN, duty=0.05, snr_db=-10.0, seed=9)
    buf = torch.empty(nsteps * n, dtype=torch.complex64, device="cuda")
    graph = g.capture(buf, nsteps)
    launches = 3
    for _ in range(launches):
        sim.generate(nsteps * n, out=buf)
        a.filter_blocks(buf, nsteps)
        graph.launch()
        torch.cuda.synchronize()
    oa = np.zeros((len(dms), B, a.M), np.complex64)
    og = np.zeros_like(oa)
    a.get_output(oa)
    g.get_output(og)
    a.synchronize()
    g.synchronize()
    assert np.array_equal(oa, og)
    pa, sa, ca = fa.read()
    pg, sg, cg = fg.read()
    assert np.abs(ca.astype(np.int64) - cg.astype(np.int64)).sum() <= 2 * len(dms)
    assert rel_l2(sg, sa) < 1e-6
    assert a.steps == g.steps == launches * nsteps


def test_graph_capture_refuses_what_it_cannot_replay(eng):
    torch = pytest.importorskip("torch")
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    m = eng.MsosmGpuBatch(bw, [100.0, 120.0], f0).initialize(1 << 18, 4, eng.IN_C64, eng.OUT_C64)
    rp = m.ring_blocks // 4
    period = rp * 2 // np.gcd(rp, 2)
    buf = torch.zeros(period * 4 * m.M, dtype=torch.complex64, device="cuda")
    with pytest.raises(eng.MsosmError):
        m.capture(buf, period + 1)  # not a multiple of the ring's period
    with pytest.raises(eng.MsosmError):
        m.capture(np.zeros(period * 4 * m.M, np.complex64), period)  # host input
    small = eng.MsosmGpuBatch(bw, [1.0], f0).initialize(1 << 12, 4, eng.IN_C64, eng.OUT_C64)
    with pytest.raises(eng.MsosmError):
        small.capture(buf, 2)  # below the persistent transform's sizes
    g = m.capture(buf, period)  # and the handle still processes normally afterwards
    m.filter_block(buf[:4 * m.M])
    m.synchronize()
    assert m.steps == 1
    del g
