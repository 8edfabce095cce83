"""DM refinement on the GPU (pymsosm.refine through the C ABI) -- the differentiation
workload's shape at reduced size (GPU):

* the comb sharpness of one many-DM pass against the FP64 oracle's;
* the smoothed objective's derivative against central differences with step 1e-3 on
  engine data;
* 8 simulated sources (16 MHz at 1392 MHz, 2 ms period, 2 % Gaussian pulse, -10 dB
  per-sample SNR, lengths 2^20..2^22, true DMs uniform in 10..300, guesses 0.5 DM off)
  refined in 20 steps each to within 0.1 DM (RMS error reported).
"""
from __future__ import annotations

import numpy as np
import pytest

from pymsosm import refine as R

pytestmark = pytest.mark.gpu

BW, F0, PERIOD, K = np.float32(16e6), np.float32(1392e6), np.float32(0.002), 256


def _source(eng, dm, n, seed):
    return eng.Simulator(BW, F0, np.float32(dm), PERIOD, kind=eng.SIM_GAUSSIAN, duty=0.02, snr_db=-10.0,
                         seed=seed).generate(n)


def test_comb_sharpness_matches_oracle(eng, orc):
    x = _source(eng, 150.0, 1 << 20, 11)
    comb = np.array([149.5, 149.9, 150.0, 150.1, 150.5], np.float32)
    S = R.comb_sharpness(x, BW, F0, comb, PERIOD, K)
    plan0 = orc.Plan(BW, F0, comb, 0, batch=1, with_response=False)
    B = plan0.delaycount + 1
    plan = orc.Plan(BW, F0, comb, 0, batch=B)
    om = orc.Msosm(plan, B, fp64=True)
    n = B * plan.M
    outs = [om.process(x[s * n:(s + 1) * n]) for s in range(len(x) // n)]
    y = np.concatenate(outs[1:], axis=1).reshape(len(comb), -1)
    dt = 1.0 / float(BW)
    ref = []
    for q in range(len(comb)):
        s_ = np.zeros(K)
        c_ = np.zeros(K, np.uint64)
        orc.fold(orc.intensity1(y[q]), K, 0.0, dt, float(PERIOD), s_, c_)
        p = orc.fold_finalize(s_, c_).astype(np.float64)
        p -= p.mean()
        ref.append(float((p * p).sum()))
    ref = np.array(ref)
    assert np.abs(S - ref).max() <= 1e-4 * ref.max()
    assert int(np.argmax(S)) == int(np.argmax(ref))


def test_smoothed_objective_derivative_on_engine_data(eng):
    x = _source(eng, 80.0, 1 << 20, 12)
    comb = 80.0 + 0.05 * np.arange(-20, 21)
    S = R.comb_sharpness(x, BW, F0, comb, PERIOD, K)
    h = 1e-3
    for d in (79.6, 79.95, 80.3):
        _, g, _ = R.smoothed_sharpness(d, comb, S, 0.1)
        fp, _, _ = R.smoothed_sharpness(d + h, comb, S, 0.1)
        fm, _, _ = R.smoothed_sharpness(d - h, comb, S, 0.1)
        assert abs(g - (fp - fm) / (2 * h)) <= 1e-3 * abs(g)


def test_refinement_converges_on_simulated_sources(eng):
    rng = np.random.default_rng(5)
    n_src = 8
    lengths = np.exp2(rng.uniform(20, 22, n_src)).astype(np.int64)
    true = rng.uniform(10, 300, n_src)
    guess = true + np.where(rng.random(n_src) < 0.5, -0.5, 0.5)
    err = []
    for i in range(n_src):
        x = _source(eng, true[i], int(lengths[i]), 100 + i)
        est, tr = R.refine_dm(x, BW, F0, guess[i], PERIOD, K)
        assert len(tr.dm) == 20
        err.append(est - true[i])
    err = np.array(err)
    print("refinement errors (DM):", np.round(err, 4), "RMS", float(np.sqrt(np.mean(err ** 2))))
    assert np.abs(err).max() < 0.1
