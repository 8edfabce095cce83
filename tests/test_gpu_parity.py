"""GPU parity: the engine through its C ABI against the FP64 oracle.

Gate (the benchmark spec): <= 1e-4 relative L2 on the dedispersed float series versus
the FP64 MS-OSM oracle with the same M, segmentation and response, and the same
folded-profile peak bin.  Integer work (delay maps, counts) is bit-exact.
Warm-up outputs -- the first delaycount+1 windows, which read spectra from before
the stream started -- are excluded, as the reference leaves them undefined.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import expand_runs, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4  # relative L2, FP32 engine vs FP64 oracle


def _engine(eng, bw, f0, dms, fftpoint, B, in_format, out_mode=1):
    m = eng.MsosmGpuBatch(bw, dms, f0)
    m.initialize(fftpoint, B, in_format, out_mode)
    return m


def _run_engine(m, chunks, out_dtype=np.complex64):
    outs = []
    for c in chunks:
        m.filter_block(np.ascontiguousarray(c))
        o = np.zeros((m.num_dms, m.batch, m.M), out_dtype)
        m.get_output(o)
        m.synchronize()
        outs.append(o)
    return outs


def _run_oracle(orc, plan, B, chunks_c):
    om = orc.Msosm(plan, B, fp64=True)
    return [om.process(c) for c in chunks_c]


def _compare_stream(got, ref, warm_windows):
    """rel-L2 per DM over all post-warm-up windows."""
    g = np.concatenate(got, axis=1)
    r = np.concatenate(ref, axis=1)
    errs = []
    for d in range(g.shape[0]):
        errs.append(rel_l2(g[d, warm_windows:], r[d, warm_windows:]))
    return max(errs)


SMALL = [
    # (name, bw, f0, dms, fftpoint, B, steps)
    ("small_4mhz_dm1to3", 4e6, 400e6, [1.0, 2.0, 3.0], 0, 4, 5),
    ("small_8mhz_dm0p5to8", 8e6, 600e6, [0.5, 1.0, 2.5, 4.0, 8.0], 0, 3, 6),
    ("psrdada_like_16mhz", 16e6, 1000e6, [5.0, 20.0], 0, 4, 3),
    ("dm0_and_1_f8192", 4e6, 400e6, [0.0, 1.0], 8192, 2, 4),
]


@pytest.mark.parametrize("case", SMALL, ids=[c[0] for c in SMALL])
def test_stream_c64_matches_oracle(eng, orc, case):
    name, bw, f0, dms, fftpoint, B, steps = case
    bw, f0 = np.float32(bw), np.float32(f0)
    m = _engine(eng, bw, f0, dms, fftpoint, B, eng.IN_C64)
    plan = orc.Plan(bw, f0, dms, fftpoint, batch=B)
    assert (m.M, m.delaycount, m.ring_blocks) == (plan.M, plan.delaycount, plan.fbs)
    for i in range(len(dms)):
        np.testing.assert_array_equal(m.delay_points(i), plan.delays[i])
        assert rel_l2(m.response(i), plan.H[i]) < 2e-7
    rng = np.random.default_rng(11)
    n = B * m.M
    chunks = [(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64) for _ in range(steps)]
    got = _run_engine(m, chunks)
    ref = _run_oracle(orc, plan, B, chunks)
    err = _compare_stream(got, ref, plan.delaycount + 1)
    assert err < TOL, err
    # and the windows before the ring filled are still finite and reproducible (zeroed ring)
    assert np.isfinite(np.concatenate(got, axis=1)).all()


def test_input_formats_u16_and_i8(eng, orc):
    bw, f0, dms, B, steps = np.float32(8e6), np.float32(600e6), [1.0, 4.0], 2, 4
    plan = orc.Plan(bw, f0, dms, 0, batch=B)
    n = B * plan.M
    rng = np.random.default_rng(5)
    # uint16 offset binary including the "no data" code 0
    raw16 = [rng.integers(0, 65536, n, dtype=np.uint32) | (rng.integers(0, 65536, n, dtype=np.uint32) << 16)
             for _ in range(steps)]
    raw16[0][:17] = 0
    m = _engine(eng, bw, f0, dms, 0, B, eng.IN_U16)
    got = _run_engine(m, raw16)
    ref = _run_oracle(orc, plan, B, [orc.decode_u16(r) for r in raw16])
    assert _compare_stream(got, ref, plan.delaycount + 1) < TOL
    # int8 interleaved I/Q
    raw8 = [rng.integers(-127, 128, 2 * n).astype(np.int8) for _ in range(steps)]
    m8 = _engine(eng, bw, f0, dms, 0, B, eng.IN_I8)
    got8 = _run_engine(m8, raw8)
    ref8 = _run_oracle(orc, plan, B, [orc.decode_i8(r) for r in raw8])
    assert _compare_stream(got8, ref8, plan.delaycount + 1) < TOL


def test_u16_output_matches_encoding_of_oracle(eng, orc):
    """discardSamplesToUint16 output: equal to the oracle's encoding except where
    FP32 and FP64 round to different integers (|diff| <= 1 LSB, rare)."""
    bw, f0, dms, B, steps = np.float32(4e6), np.float32(400e6), [1.0, 3.0], 4, 3
    plan = orc.Plan(bw, f0, dms, 0, batch=B)
    n = B * plan.M
    rng = np.random.default_rng(6)
    chunks = [((rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 300).astype(np.complex64) for _ in range(steps)]
    m = _engine(eng, bw, f0, dms, 0, B, eng.IN_C64, eng.OUT_U16)
    got = _run_engine(m, chunks, np.uint32)
    ref = _run_oracle(orc, plan, B, chunks)
    w = plan.delaycount + 1
    g = np.concatenate(got, axis=1)[:, w:].ravel()
    r = orc.encode_u16(np.concatenate(ref, axis=1)[:, w:].ravel().astype(np.complex64))
    gx, gy = (g & 0xFFFF).astype(np.int64), (g >> 16).astype(np.int64)
    rx, ry = (r & 0xFFFF).astype(np.int64), (r >> 16).astype(np.int64)
    assert np.abs(gx - rx).max() <= 1 and np.abs(gy - ry).max() <= 1
    assert np.mean(g == r) > 0.999


@pytest.mark.parametrize("L", list(range(8, 23)))
def test_every_fft_size(eng, orc, L):
    """Each (N1, N2) tile instantiation, F = 2^8 .. 2^22: DM 0 must reproduce the
    input exactly (identity filter) and a small DM must match the oracle."""
    F = 1 << L
    bw, f0 = np.float32(2e6), np.float32(300e6)
    B, steps = (2, 3) if L < 20 else (1, 2)
    dms = [0.0] if L < 10 else [0.0, 0.05]
    m = _engine(eng, bw, f0, dms, F, B, eng.IN_C64)
    assert m.fftpoint == F
    rng = np.random.default_rng(L)
    n = B * m.M
    chunks = [(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64) for _ in range(steps)]
    got = _run_engine(m, chunks)
    x = np.concatenate(chunks)
    y0 = np.concatenate([o[0].reshape(-1) for o in got])
    assert rel_l2(y0, x) < 1e-5
    if len(dms) > 1:
        plan = orc.Plan(bw, f0, dms, F, batch=B)
        ref = _run_oracle(orc, plan, B, chunks)
        assert _compare_stream(got, ref, plan.delaycount + 1) < TOL


def test_fused_fold_matches_oracle(eng, orc):
    """|x|^2 phase fold fused into the inverse transform vs folding the oracle series."""
    bw, f0, dms, B, steps = np.float32(4e6), np.float32(400e6), [1.0, 2.0, 3.0], 4, 6
    K, period = 64, np.float32(0.0031)
    plan = orc.Plan(bw, f0, dms, 0, batch=B)
    n = B * plan.M
    rng = np.random.default_rng(7)
    chunks = [(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64) for _ in range(steps)]
    m = _engine(eng, bw, f0, dms, 0, B, eng.IN_C64, eng.OUT_NONE)
    fold = eng.FoldGpu(period, bw, n, K, len(dms))
    m.attach_fold(fold)
    for c in chunks:
        m.filter_block(c)
    m.synchronize()
    folded, sums, cnts = fold.read()
    ref = _run_oracle(orc, plan, B, chunks)
    dt = 1.0 / float(bw)
    for d in range(len(dms)):
        s = np.zeros(K)
        c_ = np.zeros(K, np.uint64)
        t0 = 0.0
        for o in ref:
            inten = orc.intensity1(o[d].reshape(-1).astype(np.complex64))
            orc.fold(inten, K, t0, dt, float(period), s, c_)
            t0 += n * dt
        moved = int(np.abs(cnts[d].astype(np.int64) - c_.astype(np.int64)).sum())
        prof = orc.fold_finalize(s, c_)
        print(f"fused fold vs FP64 foldDataPhase, trial {d}: {moved} sample(s) in another bin of "
              f"{int(c_.sum())}, sums rel-L2 {rel_l2(sums[d], s):.2e}, profile rel-L2 {rel_l2(folded[d], prof):.2e}")
        assert int(cnts[d].sum()) == int(c_.sum())
        assert moved <= 2
        assert rel_l2(sums[d], s) < TOL
        assert rel_l2(folded[d], prof) < TOL
        assert int(np.argmax(folded[d])) == int(np.argmax(prof))


def test_standalone_fold_1pol_2pol(eng, orc):
    import torch

    size, S, K = 3 * 4096 + 77, 2, 100
    period, fs = np.float32(0.0013), np.float32(4e6)
    rng = np.random.default_rng(8)
    a = (rng.standard_normal((S, size)) + 1j * rng.standard_normal((S, size))).astype(np.complex64)
    b = (rng.standard_normal((S, size)) + 1j * rng.standard_normal((S, size))).astype(np.complex64)
    a[0, :5] = 0
    da = torch.from_numpy(a.view(np.float32)).cuda()
    db = torch.from_numpy(b.view(np.float32)).cuda()
    dt = 1.0 / float(fs)
    for two in (False, True):
        f = eng.FoldGpu(period, fs, size, K, S)
        for call in range(3):
            f.accumulate(da, db if two else None)
        torch.cuda.synchronize()
        folded, sums, cnts = f.read()
        for s in range(S):
            inten = orc.intensity2(a[s], b[s]) if two else orc.intensity1(a[s])
            rs = np.zeros(K)
            rc = np.zeros(K, np.uint64)
            for call in range(3):
                orc.fold(inten, K, call * size * dt, dt, float(period), rs, rc)
            assert np.abs(cnts[s].astype(np.int64) - rc.astype(np.int64)).sum() <= 2
            assert rel_l2(sums[s], rs) < 1e-5
            assert int(np.argmax(folded[s])) == int(np.argmax(orc.fold_finalize(rs, rc)))


def test_osm_matches_oracle(eng, orc, golden_osm):
    c = golden_osm["osm_small_dm3"]
    bw, f0, dm = np.float32(c["bw"]), np.float32(c["f0"]), c["dm"]
    m = eng.OsmGpuBatch(bw, dm, f0).initialize(0, 2, eng.IN_C64, eng.OUT_C64)
    assert m.M == c["M"] and m.nd[0] == c["nd"]
    assert not m.delay_points(0).any()
    plan = orc.Plan(bw, f0, [dm], 2 * m.M, batch=2)
    plan.delays[:] = 0
    plan.delaycount = 1
    rng = np.random.default_rng(9)
    n = 2 * m.M
    chunks = [(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64) for _ in range(3)]
    got = _run_engine(m, chunks)
    ref = _run_oracle(orc, plan, 2, chunks)
    assert _compare_stream(got, ref, 1) < TOL


def test_osm_at_the_largest_transform(eng, orc):
    """Plain overlap-save at the many-DM grid's top end: 64 MHz at 1368 MHz, DM 200,
    Nd = 2.48e6, so Prepare_OSM's order gives F = 2^24 (osm_prepare.cpp:17-30); the
    series against the FP64 oracle after the first window, and DM 0 as the identity."""
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    m = eng.OsmGpuBatch(bw, np.float32(200.0), f0).initialize(0, 1, eng.IN_C64, eng.OUT_C64)
    assert m.fftpoint == 1 << 24 and m.nd[0] == orc.osm_nd(bw, np.float32(200.0), f0)
    plan = orc.Plan(bw, f0, [200.0], m.fftpoint, batch=1)
    plan.delays[:] = 0
    plan.delaycount = 1
    rng = np.random.default_rng(24)
    chunks = [(rng.standard_normal(m.M) + 1j * rng.standard_normal(m.M)).astype(np.complex64) for _ in range(3)]
    got = _run_engine(m, chunks)
    ref = _run_oracle(orc, plan, 1, chunks)
    err = _compare_stream(got, ref, 1)
    print(f"OSM F = 2^24, DM 200: rel-L2 vs FP64 oracle {err:.2e}")
    assert err < TOL
    ident = eng.OsmGpuBatch(bw, np.float32(0.0), f0).initialize(1 << 24, 1, eng.IN_C64, eng.OUT_C64)
    out = _run_engine(ident, chunks)
    for c, o in zip(chunks, out):
        assert rel_l2(o.reshape(-1), c) < 1e-6


def test_c1_single_dm_full_size(eng, orc):
    """Single-DM workload at full size: 16 MHz at 1400 MHz, DM 50, 2^22 complex64
    samples of a dispersed pulsar (period 33 ms, 5 % duty, -10 dB), F = 2^16,
    folded into 256 bins.  Series within 1e-4 of the FP64 oracle, same peak bin."""
    from pymsosm.simulate import pulsar_signal

    bw, f0, dm = np.float32(16e6), np.float32(1392e6), 50.0
    N, B, K, period = 1 << 22, 32, 256, np.float32(0.033)
    x = pulsar_signal(N, float(bw), float(f0), dm, float(period), seed=1)
    m = _engine(eng, bw, f0, [dm], 1 << 16, B, eng.IN_C64, eng.OUT_C64)
    steps = N // (B * m.M)
    fold = eng.FoldGpu(period, bw, B * m.M, K, 1)
    m.attach_fold(fold)
    chunks = [x[s * B * m.M:(s + 1) * B * m.M] for s in range(steps)]
    got = _run_engine(m, chunks)
    plan = orc.Plan(bw, f0, [dm], 1 << 16, batch=B)
    ref = _run_oracle(orc, plan, B, chunks)
    assert _compare_stream(got, ref, plan.delaycount + 1) < TOL
    folded, _, _ = fold.read()
    s = np.zeros(K)
    c_ = np.zeros(K, np.uint64)
    dt = 1.0 / float(bw)
    for i, o in enumerate(ref):
        orc.fold(orc.intensity1(o[0].reshape(-1).astype(np.complex64)), K, i * B * m.M * dt, dt, float(period), s, c_)
    prof = orc.fold_finalize(s, c_)
    assert rel_l2(folded[0], prof) < TOL
    assert int(np.argmax(folded[0])) == int(np.argmax(prof))


def test_c2_full_size(eng, orc, golden_plans):
    """Many-DM workload at full size: 64 MHz at 1400 MHz, 512 DMs in 0..200,
    F = 2^18, 2^26 complex64 samples with a pulsar injected at DM 123.4, 512 bins.

    * all 512 trials run fold-only (fused fold), as the throughput benchmark does;
    * DMs 0, 123.68 (grid point nearest 123.4) and 200 run again with series
      output: they match the FP64 oracle over the whole stream, DM 0 returns the
      input, and their folds equal the 512-trial run's rows (DM batching and
      launch chunking do not change any trial);
    * the dedispersed pulse at the injected DM peaks far above DM 0's smeared one.
    """
    from pymsosm.simulate import pulsar_signal

    c = golden_plans["c2_512dm_f262144"]
    bw, f0 = np.float32(c["bw"]), np.float32(c["f0"])
    dms = np.array(c["dms"], np.float32)
    N, B, K, period = 1 << 26, 32, 512, np.float32(0.033)
    x = pulsar_signal(N, float(bw), float(f0), 123.4, float(period), seed=2)

    full = _engine(eng, bw, f0, dms, 1 << 18, B, eng.IN_C64, eng.OUT_NONE)
    assert full.delaycount == c["delaycount"] and full.M == c["M"]
    step_n = B * full.M
    steps = N // step_n
    fold_all = eng.FoldGpu(period, bw, step_n, K, len(dms))
    full.attach_fold(fold_all)
    full.filter_blocks(x, steps)
    full.synchronize()
    prof_all, sums_all, cnts_all = fold_all.read()

    pick = [0, int(np.argmin(np.abs(dms - 123.4))), 511]
    sub = _engine(eng, bw, f0, dms[pick], 1 << 18, B, eng.IN_C64, eng.OUT_C64)
    assert sub.M == full.M
    for k, i in enumerate(pick[1:], start=1):
        np.testing.assert_array_equal(sub.delay_points(k), expand_runs(c["delay_runs"][i], sub.fftpoint))
    fold_sub = eng.FoldGpu(period, bw, step_n, K, len(pick))
    sub.attach_fold(fold_sub)
    chunks = [x[s * step_n:(s + 1) * step_n] for s in range(steps)]
    got = _run_engine(sub, chunks)
    _, sums_sub, cnts_sub = fold_sub.read()
    np.testing.assert_array_equal(cnts_sub, cnts_all[pick])
    assert rel_l2(sums_sub, sums_all[pick]) < 1e-6

    y0 = np.concatenate([g[0].reshape(-1) for g in got])
    assert rel_l2(y0, x[:y0.size]) < 1e-5
    plan = orc.Plan(bw, f0, dms[pick], 1 << 18, batch=B)
    ref = _run_oracle(orc, plan, B, chunks)
    assert _compare_stream(got, ref, plan.delaycount + 1) < TOL

    def snr(p):
        base = np.median(p)
        return (p.max() - base) / (1.4826 * np.median(np.abs(p - base)))

    s_all = np.array([snr(p) for p in prof_all])
    assert s_all[pick[1]] > 3 * s_all[0]
    assert abs(float(dms[int(np.argmax(s_all))]) - 123.4) < 10.0


def test_linearity_at_full_size(eng):
    """Size-independent property at the many-DM workload's F = 2^18: the streaming filter
    is linear in its input (zero-initialised state included), for every DM trial."""
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    dms = [50.0, 123.4, 200.0]
    B, steps = 8, 3
    rng = np.random.default_rng(17)
    runs = []
    xs = [[(rng.standard_normal(B << 17) + 1j * rng.standard_normal(B << 17)).astype(np.complex64)
           for _ in range(steps)] for _ in range(2)]
    combo = [(2.0 * a - 3.0 * b).astype(np.complex64) for a, b in zip(*xs)]
    for chunks in (xs[0], xs[1], combo):
        m = _engine(eng, bw, f0, dms, 1 << 18, B, eng.IN_C64)
        runs.append(np.concatenate(_run_engine(m, chunks), axis=1))
    expect = 2.0 * runs[0].astype(np.complex128) - 3.0 * runs[1].astype(np.complex128)
    for d in range(len(dms)):
        assert rel_l2(runs[2][d], expect[d]) < 1e-5


@pytest.mark.parametrize("group", [4, 8, 13, 32])
def test_transform_order_does_not_change_outputs(eng, group):
    """msosm_set_launch_shape's DM grouping (window-major groups, the last one partial)
    and one CTA per SM give the DM-major order's series bit for bit, and its folds to
    the fused fold's float-sum order."""
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    dms = np.linspace(20.0, 180.0, 13).astype(np.float32)
    F, B, K = 1 << 18, 4, 128
    procs, folds = [], []
    for g, ctas in ((1, 0), (group, 0), (group, 1)):
        m = eng.MsosmGpuBatch(bw, dms, f0).initialize(F, B, eng.IN_C64, eng.OUT_C64).set_launch_shape(ctas, g)
        f = eng.FoldGpu(np.float32(0.0047), bw, B * m.M, K, len(dms))
        m.attach_fold(f)
        procs.append(m)
        folds.append(f)
    rng = np.random.default_rng(group)
    outs = [np.zeros((len(dms), B, procs[0].M), np.complex64) for _ in procs]
    for s in range(3):
        x = (rng.standard_normal(B * procs[0].M) + 1j * rng.standard_normal(B * procs[0].M)).astype(np.complex64)
        for m, o in zip(procs, outs):
            m.filter_block(x)
            m.get_output(o)
            m.synchronize()
        assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    ref = folds[0].read()
    for f in folds[1:]:
        _, sums, cnts = f.read()
        assert np.array_equal(cnts, ref[2])
        assert rel_l2(sums, ref[1]) < 1e-6
