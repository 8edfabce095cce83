"""Error of every DM trial of the many-DM workload against the FP64 oracle (GPU).

Many-DM grid at full transform size: 64 MHz at 1400 MHz, 512 DMs in 0..200, F = 2^18;
8 windows per call, 4 calls of Gaussian baseband.  Each trial's dedispersed series is
compared with the FP64 MS-OSM oracle (same M, segmentation and response) over its
post-warm-up windows, for the FP32 register transform and for the split-precision
tensor-core transform with BF16 and with FP16 hi/lo operands; the per-trial relative L2
errors are reported side by side and the worst of each must stay within the 1e-4 gate.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_every_trial_of_the_many_dm_grid(eng, orc, golden_plans):
    c = golden_plans["c2_512dm_f262144"]
    bw, f0 = np.float32(c["bw"]), np.float32(c["f0"])
    dms = np.array(c["dms"], np.float32)
    B, calls = 8, 4
    precs = {"fp32": eng.PREC_FP32, "bf16x3": eng.PREC_BF16X3, "fp16x3": eng.PREC_FP16X3}
    procs = {k: eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 18, B, eng.IN_C64, eng.OUT_C64).set_precision(p)
             for k, p in precs.items()}
    m = procs["fp32"]
    plan = orc.Plan(bw, f0, dms, 1 << 18, batch=B)
    assert plan.delaycount == m.delaycount == c["delaycount"]
    om = orc.Msosm(plan, B, fp64=True)
    dc = m.delaycounts()
    err2 = {k: np.zeros(len(dms)) for k in procs}
    ref2 = np.zeros(len(dms))
    rng = np.random.default_rng(23)
    out = np.zeros((len(dms), B, m.M), np.complex64)
    for s in range(calls):
        x = (rng.standard_normal(B * m.M) + 1j * rng.standard_normal(B * m.M)).astype(np.complex64)
        r = om.process(x)
        for k, p in procs.items():
            p.filter_block(x)
            p.get_output(out)
            p.synchronize()
            for d in range(len(dms)):
                w0 = max(0, dc[d] + 1 - s * B)  # windows of this call before trial d's ring filled
                if w0 >= B:
                    continue
                diff = out[d, w0:].astype(np.complex128) - r[d, w0:]
                err2[k][d] += float(np.vdot(diff, diff).real)
                if k == "fp32":
                    ref2[d] += float(np.vdot(r[d, w0:], r[d, w0:]).real)
    assert np.all(ref2 > 0)
    worst = {}
    for k in procs:
        rel = np.sqrt(err2[k] / ref2)
        worst[k] = rel.max()
        print(f"{k}: per-trial rel-L2 vs FP64 over {len(dms)} trials: median {np.median(rel):.2e}, "
              f"90th pct {np.percentile(rel, 90):.2e}, max {rel.max():.2e} (DM {dms[int(np.argmax(rel))]:.2f})")
    assert max(worst.values()) < 1e-4, worst
