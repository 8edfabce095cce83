"""The 2-pol int8 batching configuration at reduced length (GPU).

Shape of the configuration: 2-pol psrdada-style int8 I/Q baseband (Gaussian,
sigma 20, clipped to [-127, 127]), 128 MHz at 820 MHz centre, DMs log-uniform in
1..1000 (sorted), which forces F = 2^20 (M_min of DM ~1000 is 2^19).  Here: 2^22
samples per pol and 48 of the trials, so the FP64 oracle can follow; the engine
runs both pols through the int8 path and folds sqrt(|a|^2+|b|^2) per DM, both as the
reference does (series out, then the 2-pol fold) and fused (msosm_attach_fold_pol2).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_two_pol_int8_f2_20(eng, orc):
    rng = np.random.default_rng(4)
    dms_all = np.sort(np.exp(rng.uniform(np.log(1.0), np.log(1000.0), 1024))).astype(np.float32)
    dms = dms_all[::22][:48]
    dms = np.concatenate([dms, dms_all[-1:]])  # keep the largest DM: it sets M
    bw, f0 = np.float32(128e6), np.float32(756e6)
    B = 2
    N = 1 << 22
    pols = []
    for p in range(2):
        iq = np.clip(np.round(rng.normal(0.0, 20.0, 2 * N)), -127, 127).astype(np.int8)
        pols.append(iq)
    ms = [eng.MsosmGpuBatch(bw, dms, f0).initialize(0, B, eng.IN_I8, eng.OUT_C64) for _ in range(2)]
    fus = [eng.MsosmGpuBatch(bw, dms, f0).initialize(0, B, eng.IN_I8, eng.OUT_NONE) for _ in range(2)]
    assert ms[0].fftpoint == 1 << 20 and ms[0].M == 1 << 19
    plan = orc.Plan(bw, f0, dms, 0, batch=B)
    assert plan.M == ms[0].M and plan.delaycount == ms[0].delaycount
    step = B * ms[0].M
    K, period = 256, np.float32(0.0071)
    fold = eng.FoldGpu(period, bw, step, K, len(dms))
    fold_fus = eng.FoldGpu(period, bw, step, K, len(dms))
    fus[0].attach_fold_pol2(fus[1], fold_fus)
    pick = [0, len(dms) // 2, len(dms) - 1]
    om = [orc.Msosm(orc.Plan(bw, f0, dms[pick], 1 << 20, batch=B), B, fp64=True) for _ in range(2)]
    got = [[], []]
    ref = [[], []]
    for s in range(N // step):
        for p in range(2):
            chunk = np.ascontiguousarray(pols[p][2 * s * step:2 * (s + 1) * step])
            ms[p].filter_block(chunk)
            o = np.zeros((len(dms), B, ms[p].M), np.complex64)
            ms[p].get_output(o)
            ms[p].synchronize()
            got[p].append(o[pick])
            ref[p].append(om[p].process(orc.decode_i8(chunk)))
        fold.accumulate(ms[0].get_output_pointer(), ms[1].get_output_pointer())
        for p in range(2):
            fus[p].filter_block(np.ascontiguousarray(pols[p][2 * s * step:2 * (s + 1) * step]))
    w = plan.delaycount + 1  # windows before the ring filled
    for p in range(2):
        g = np.concatenate(got[p], axis=1)
        r = np.concatenate(ref[p], axis=1)
        for k in range(len(pick)):
            assert rel_l2(g[k, w:], r[k, w:]) < 1e-4
    folded, sums, cnts = fold.read()
    assert cnts.sum() > 0 and np.isfinite(folded).all()
    # the fused 2-pol fold (no series written) folds the same intensities
    _, fsums, fcnts = fold_fus.read()
    assert np.abs(fcnts.astype(np.int64) - cnts.astype(np.int64)).sum() <= 2 * len(dms)
    assert rel_l2(fsums, sums) < 1e-5
    # the 2-pol fold of the picked trials equals folding the engine's own series
    dt = 1.0 / float(bw)
    for k, d in enumerate(pick):
        s_ = np.zeros(K)
        c_ = np.zeros(K, np.uint64)
        for s in range(N // step):
            a = got[0][s][k].reshape(-1)
            b = got[1][s][k].reshape(-1)
            orc.fold(orc.intensity2(a, b), K, s * step * dt, dt, float(period), s_, c_)
        assert np.abs(cnts[d].astype(np.int64) - c_.astype(np.int64)).sum() <= 2
        assert rel_l2(sums[d], s_) < 1e-5


def test_autotune_picks_a_valid_size_and_caches(eng, tmp_path):
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    dms = np.linspace(0.0, 200.0, 64).astype(np.float32)
    cache = tmp_path / "tune.json"
    F, rate = eng.autotune(bw, f0, dms, 8, eng.IN_C64, 1 << 16, 1 << 20, 2, cache=cache)
    mmin = eng.plan_min_order(eng.plan_nd(bw, f0, dms))
    assert F >= 2 * mmin and F <= 1 << 20 and (F & (F - 1)) == 0
    assert rate > 0
    assert eng.autotune(bw, f0, dms, 8, eng.IN_C64, 1 << 16, 1 << 20, 2, cache=cache) == (F, rate)


def test_fused_two_pol_fold_matches_the_standalone_fold(eng):
    """msosm_attach_fold_pol2 folds sqrt(|a|^2 + |b|^2) inside the second polarisation's
    transform; it must equal the reference-shaped path (both series out, Fold_GPU's 2-pol
    intensity) on the same int8 baseband."""
    rng = np.random.default_rng(9)
    bw, f0 = np.float32(32e6), np.float32(800e6)
    dms = np.sort(rng.uniform(5.0, 60.0, 6)).astype(np.float32)
    B, K, period, steps = 4, 256, np.float32(0.0031), 3
    ref = [eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 16, B, eng.IN_I8, eng.OUT_C64) for _ in range(2)]
    fus = [eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 16, B, eng.IN_I8, eng.OUT_NONE) for _ in range(2)]
    M = ref[0].M
    fold_ref = eng.FoldGpu(period, bw, B * M, K, len(dms))
    fold_fus = eng.FoldGpu(period, bw, B * M, K, len(dms))
    fus[0].attach_fold_pol2(fus[1], fold_fus)
    for s in range(steps):
        a = np.clip(np.round(rng.normal(0, 20, 2 * B * M)), -127, 127).astype(np.int8)
        b = np.clip(np.round(rng.normal(0, 20, 2 * B * M)), -127, 127).astype(np.int8)
        ref[0].filter_block(a)
        ref[1].filter_block(b)
        fold_ref.accumulate(ref[0].get_output_pointer(), ref[1].get_output_pointer())
        fus[0].filter_block(a)
        fus[1].filter_block(b)
    _, s_ref, c_ref = fold_ref.read()
    _, s_fus, c_fus = fold_fus.read()
    assert int(c_fus.sum()) == len(dms) * steps * B * M
    assert np.abs(c_fus.astype(np.int64) - c_ref.astype(np.int64)).sum() <= 2 * len(dms)
    assert rel_l2(s_fus, s_ref) < 1e-5


def test_fused_two_pol_fold_rejects_series_output(eng):
    bw, f0, dms = np.float32(32e6), np.float32(800e6), [10.0, 20.0]
    a = eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 16, 4, eng.IN_I8, eng.OUT_C64)
    b = eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 16, 4, eng.IN_I8, eng.OUT_NONE)
    fold = eng.FoldGpu(np.float32(0.0031), bw, 4 * a.M, 64, len(dms))
    with pytest.raises(eng.MsosmError):
        a.attach_fold_pol2(b, fold)


def test_two_pol_int8_full_size(eng, orc):
    """The batching configuration at full size: 2 x 2^28 int8 samples, all 1024
    log-uniform DMs, F = 2^20.  The fused 2-pol fold (no series) of every trial against
    the reference-shaped path (series out, then the 2-pol fold); the series of 16 trials
    spread over the grid (the widest, delaycount 472, included) against the FP64 oracle
    over the last 16 windows of the 512, all past every trial's ring warm-up."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    dms = np.sort(np.exp(rng.uniform(np.log(1.0), np.log(1000.0), 1024))).astype(np.float32)
    bw, f0 = np.float32(128e6), np.float32(756e6)
    B, N, K, period = 2, 1 << 28, 256, np.float32(0.0071)
    dev = torch.device("cuda")
    pols = []
    for p in range(2):
        g = torch.empty(N, dtype=torch.complex64, device=dev)
        eng.awgn(N, 0.0, 20.0, seed=40 + p, out=g)
        iq = torch.view_as_real(g).reshape(-1).round().clamp(-127, 127).to(torch.int8)
        del g
        pols.append(iq)
    torch.cuda.synchronize()
    fus = [eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 20, B, eng.IN_I8, eng.OUT_NONE) for _ in range(2)]
    ref = [eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 20, B, eng.IN_I8, eng.OUT_C64) for _ in range(2)]
    assert fus[0].M == 1 << 19 and fus[0].delaycount > 400
    step = B * fus[0].M
    fold_fus = eng.FoldGpu(period, bw, step, K, len(dms))
    fold_ref = eng.FoldGpu(period, bw, step, K, len(dms))
    fus[0].attach_fold_pol2(fus[1], fold_fus)
    pick = np.unique(np.r_[np.linspace(0, len(dms) - 1, 16).round().astype(int), len(dms) - 1])
    ser = [eng.MsosmGpuBatch(bw, dms[pick], f0).initialize(1 << 20, B, eng.IN_I8, eng.OUT_C64) for _ in range(2)]
    steps = N // step
    tail = 8  # the last 8 steps (16 windows) are compared, all past every trial's warm-up
    got = [np.zeros((len(pick), tail * step), np.complex64) for _ in range(2)]
    for s in range(steps):
        for p in range(2):
            src = pols[p][2 * s * step:2 * (s + 1) * step]
            fus[p].filter_block(src)
            ref[p].filter_block(src)
            ser[p].filter_block(src)
        fold_ref.accumulate(ref[0].get_output_pointer(), ref[1].get_output_pointer())
        if s >= steps - tail:
            for p in range(2):
                o = np.zeros((len(pick), B, ser[p].M), np.complex64)
                ser[p].get_output(o)
                ser[p].synchronize()
                j = s - (steps - tail)
                got[p][:, j * step:(j + 1) * step] = o.reshape(len(pick), -1)
    fus[1].synchronize()
    _, fsums, fcnts = fold_fus.read()
    _, rsums, rcnts = fold_ref.read()
    # every trial: the fused fold folds what the reference-shaped path folds
    assert np.abs(fcnts.astype(np.int64) - rcnts.astype(np.int64)).max() <= 2
    for d in range(len(dms)):
        assert rel_l2(fsums[d], rsums[d]) < 1e-5, d
    # the picked trials' series against the FP64 oracle after each trial's warm-up
    host = [pols[p].cpu().numpy() for p in range(2)]
    plan = orc.Plan(bw, f0, dms[pick], 1 << 20, batch=B)
    assert (steps - tail) * B > plan.delaycount + 2  # every compared window is past the warm-up
    for p in range(2):
        om = orc.Msosm(plan, B, fp64=True)
        r = np.zeros((len(pick), tail * step), np.complex128)
        for s in range(steps):
            o = om.process(orc.decode_i8(host[p][2 * s * step:2 * (s + 1) * step]), want_output=s >= steps - tail)
            if o is not None:
                j = s - (steps - tail)
                r[:, j * step:(j + 1) * step] = o.reshape(len(pick), -1)
        for k in range(len(pick)):
            assert rel_l2(got[p][k], r[k]) < 1e-4, (p, k, float(dms[pick[k]]))


def test_autotune_shape_picks_a_valid_triple(eng):
    bw, f0 = np.float32(128e6), np.float32(756e6)
    rng = np.random.default_rng(4)
    dms = np.sort(np.exp(rng.uniform(np.log(1.0), np.log(1000.0), 1024))).astype(np.float32)
    best = eng.autotune_shape(bw, f0, dms, batches=(2, 8), in_format=eng.IN_I8, min_fftpoint=1 << 16,
                              max_fftpoint=1 << 20, steps=2)
    print("autotune_shape:", best)
    assert best["fftpoint"] == 1 << 20  # the largest DM forces F = 2^20
    assert best["batch"] in (2, 8) and best["ctas_per_sm"] in (0, 1) and best["rate"] > 0
    m = eng.MsosmGpuBatch(bw, dms[:4], f0).initialize(1 << 20, 2, eng.IN_I8, eng.OUT_C64).set_launch_shape(1)
    m.filter_block(np.zeros(2 * 2 * m.M, np.int8))
    m.synchronize()
    torch = pytest.importorskip("torch")
    assert m.launch_info()["grid"] == torch.cuda.get_device_properties(0).multi_processor_count
