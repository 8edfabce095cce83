"""The GPU pulsar simulator (msosm_sim_*, msosm_awgn) through the C ABI (GPU).

* every pulse kind, with and without noise, against the numpy FP64 model of the same
  generator (oracle/oracle_sim.py) over a stream cut into uneven calls, in complex64,
  uint16 and int8;
* AWGN samples against the model's Philox / Box-Muller draws;
* the physics the generator must carry, on the single-DM workload's signal (16 MHz at
  1392 MHz, DM 50, 33 ms period, 5 % Gaussian pulse, -10 dB per-sample SNR, 2^22
  samples, F = 2^16, 256 phase bins): dedispersing at the injected DM recovers the
  pulse at phase 0.5 with high S/N, trial DMs far from it recover less.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_sim as osim
from conftest import rel_l2

pytestmark = pytest.mark.gpu

C1 = dict(bw=np.float32(16e6), f0=np.float32(1392e6), dm=np.float32(50.0), period=np.float32(0.033))


@pytest.mark.parametrize("kind,snr", [(0, None), (1, -10.0), (2, None)])
def test_generator_matches_numpy_model(eng, kind, snr):
    bw, f0, dm, period = C1["bw"], C1["f0"], C1["dm"], C1["period"]
    sim = eng.Simulator(bw, f0, dm, period, kind=kind, duty=0.05, snr_db=snr, seed=7)
    assert sim.nd == osim.smear(bw, dm, f0) == 38719
    assert sim.period_samples == osim.period_samples(bw, period) == 528000
    sizes = [400_000, 700_001, 399_999]
    got = np.concatenate([sim.generate(n) for n in sizes])
    assert sim.position == sum(sizes)
    ref = osim.generate(sum(sizes), bw, f0, dm, period, kind=kind, duty=0.05, snr_db=snr, seed=7)
    err = rel_l2(got, ref)
    print(f"kind {kind} snr {snr}: rel-L2 vs FP64 model {err:.2e}")
    assert err < 2e-5
    if snr is not None:
        # encoded forms of the same stream: uint16 within one code (truncation edges),
        # int8 within one step, nearly all identical
        u16 = eng.Simulator(bw, f0, dm, period, kind=kind, duty=0.05, snr_db=snr, seed=7).generate(
            sum(sizes), eng.IN_U16, 0.05)
        want = osim.encode_u16(ref * 0.05)
        for sh in (0, 16):
            d = np.abs(((u16 >> sh) & 0xFFFF).astype(np.int64) - ((want >> sh) & 0xFFFF).astype(np.int64))
            assert d.max() <= 1 and np.mean(d == 0) > 0.999
        i8 = eng.Simulator(bw, f0, dm, period, kind=kind, duty=0.05, snr_db=snr, seed=7).generate(
            sum(sizes), eng.IN_I8, 0.02)
        w8 = np.empty(2 * ref.size)
        w8[0::2], w8[1::2] = ref.real * 0.02, ref.imag * 0.02
        w8 = np.clip(np.rint(w8), -127, 127)
        d8 = np.abs(i8.astype(np.int64) - w8.astype(np.int64))
        assert d8.max() <= 1 and np.mean(d8 == 0) > 0.999


def test_generator_on_device_output(eng):
    torch = pytest.importorskip("torch")
    bw, f0, dm, period = C1["bw"], C1["f0"], C1["dm"], C1["period"]
    n = 1 << 20
    host = eng.Simulator(bw, f0, dm, period, kind=1, snr_db=-10.0, seed=3).generate(n)
    dev = torch.zeros(n, dtype=torch.complex64, device="cuda")
    eng.Simulator(bw, f0, dm, period, kind=1, snr_db=-10.0, seed=3).generate(n, out=dev)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)


def test_awgn_matches_model(eng):
    n, mean, sd = 1 << 20, 0.25, 3.0
    got = eng.awgn(n, mean, sd, seed=11, first=5)
    ref = mean * (1 + 1j) + sd * osim.normal_pairs(np.arange(5, 5 + n, dtype=np.uint64), 2, 11)
    assert np.abs(got - ref).max() < 1e-4 * sd
    assert abs(got.real.mean() - mean) < 0.02 and abs(got.real.std() - sd) < 0.02


def test_dedispersion_recovers_the_simulated_pulse(eng):
    bw, f0, dm, period = C1["bw"], C1["f0"], C1["dm"], C1["period"]
    N, F, B, K = 1 << 22, 1 << 16, 32, 256
    x = eng.Simulator(bw, f0, dm, period, kind=eng.SIM_GAUSSIAN, duty=0.05, snr_db=-10.0, seed=1).generate(N)
    assert (x != 0).all()
    dms = np.array([0.0, 25.0, 50.0, 75.0, 100.0], np.float32)
    m = eng.MsosmGpuBatch(bw, dms, f0).initialize(F, B, eng.IN_C64, eng.OUT_NONE)
    n = B * m.M
    steps = N // n
    # the first step holds every trial's ring warm-up ((delaycount + 1) * M samples with
    # partial history, fewer for smaller DMs): fold from the second step on, so that the
    # phase origin is sample n
    fold = eng.FoldGpu(period, bw, n, K, len(dms))
    for s in range(steps):
        if s == 1:
            m.attach_fold(fold)
        m.filter_block(np.ascontiguousarray(x[s * n:(s + 1) * n]))
    m.synchronize()
    prof, _, _ = fold.read()
    Np = osim.period_samples(bw, period)
    want = int(round(((0.5 - (n % Np) / Np) % 1.0) * K)) % K  # phase 0.5 of the emission
    dist = np.abs(np.arange(K) - want)
    off_pulse = np.minimum(dist, K - dist) > K // 4
    snr = []
    for d in range(len(dms)):
        p = prof[d].astype(np.float64)
        off = p[off_pulse]
        snr.append((p.max() - np.median(off)) / off.std())
    best = int(np.argmax(snr))
    peak = int(np.argmax(prof[best]))
    print("S/N per DM:", dict(zip(dms.tolist(), np.round(snr, 1))), "peak bin", peak)
    assert dms[best] == 50.0
    assert min(abs(peak - want), K - abs(peak - want)) <= 3
    assert snr[best] > 30
    # the smear at DM 50 is 7 % of the period: trials far from it lose much of the S/N
    assert snr[0] < 0.7 * snr[best] and snr[-1] < 0.7 * snr[best]


def test_simulator_refuses_bad_requests(eng):
    with pytest.raises(eng.MsosmError):
        eng.Simulator(np.float32(16e6), np.float32(1392e6), np.float32(-1.0), np.float32(0.033))
    with pytest.raises(eng.MsosmError):
        eng.Simulator(np.float32(16e6), np.float32(1392e6), np.float32(5.0), np.float32(0.001), kind=7)
    with pytest.raises(eng.MsosmError):
        eng.Simulator(np.float32(16e6), np.float32(1392e6), np.float32(5.0), np.float32(0.001),
                      kind=eng.SIM_GAUSSIAN, duty=1.5)
    s = eng.Simulator(np.float32(16e6), np.float32(1392e6), np.float32(5.0), np.float32(0.001))
    s.generate(1000)
    L = eng.lib()
    for call in (lambda: L.msosm_sim_set_seed(s._h, 3), lambda: L.msosm_sim_set_noise(s._h, 1, 0.0),
                 lambda: L.msosm_sim_set_pulse(s._h, eng.SIM_IMPULSES, 0.05)):
        with pytest.raises(eng.MsosmError, match="after the first generate"):
            s._check(call())  # the signal model is fixed once generation started
    assert s.position == 1000
    # a smear of 2^23 samples or more would need a transform above 2^24 points
    big = eng.Simulator(np.float32(128e6), np.float32(756e6), np.float32(1000.0), np.float32(0.01))
    with pytest.raises(eng.MsosmError):
        big.generate(10)
