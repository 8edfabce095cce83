"""Checkpoint/resume of the stream state and the DM derivative of folded-profile
sharpness, through the C ABI (GPU), plus the response derivative on the CPU."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

KDM = 4.15e15


# ----------------------------------------------------------------------------- CPU
def test_response_derivative_matches_oracle_and_differences(eng, orc):
    bw, f0, M = np.float32(4e6), np.float32(400e6), 2048
    for dm in (0.0, 1.7, 2.3):
        dH = eng.plan_response_derivative(bw, f0, dm, M)
        ref = orc.response_derivative(bw, f0, dm, M)
        assert rel_l2(dH, ref) < 1e-6
    # the construction is linear in the chirp, so H(dm+h)-H(dm-h) / 2h -> dH (FP64);
    # the band-edge phase moves ~6.5e3 rad per unit DM here, so the step must be tiny
    dm, h = 2.0, 1e-6
    fd = (orc.response(bw, f0, np.float32(dm + h), M) - orc.response(bw, f0, np.float32(dm - h), M)) / (
        float(np.float32(dm + h)) - float(np.float32(dm - h)))
    assert rel_l2(orc.response_derivative(bw, f0, dm, M), fd) < 1e-5


# ----------------------------------------------------------------------------- GPU
def _fold64(x, K, t0, dt, period, sums, cnts, weights=None):
    """FP64 fold of |x|^2 (or of `weights`) with the reference's phase formula."""
    i = np.arange(x.size, dtype=np.float64)
    t = t0 + i * dt
    b = np.floor(np.fmod(t / period, 1.0) * K).astype(np.int64)
    b = np.minimum(b, K - 1)
    p = np.abs(x) ** 2
    keep = p != 0
    w = p if weights is None else weights
    sums += np.bincount(b[keep], weights=w[keep], minlength=K)
    cnts += np.bincount(b[keep], minlength=K)


def _oracle_sharpness(orc, x, bw, f0, dms, fftpoint, B, period, K, with_grad=True, delays=None):
    plan = orc.Plan(bw, f0, dms, fftpoint, batch=B)
    if delays is not None:  # hold another DM's segmentation fixed
        assert delays.shape == plan.delays.shape
        plan.delays[:] = delays
        plan.delaycount = max(plan.delaycount, int(delays.max()) + 1)
    mx = orc.Msosm(plan, B, fp64=True)
    md = None
    if with_grad:
        dH = np.stack([orc.response_derivative(bw, f0, float(d), plan.M) for d in plan.dms])
        md = orc.Msosm(plan, B, fp64=True, H=dH)
    n = B * plan.M
    D = len(plan.dms)
    sx = np.zeros((D, K))
    sg = np.zeros((D, K))
    cx = np.zeros((D, K))
    dt = 1.0 / float(np.float32(bw))
    for s in range(len(x) // n):
        c = x[s * n:(s + 1) * n]
        ox = mx.process(c)
        od = md.process(c) if md else None
        for d in range(D):
            xs = ox[d].reshape(-1)
            _fold64(xs, K, s * n * dt, dt, float(np.float32(period)), sx[d], cx[d])
            if md:
                ds = od[d].reshape(-1)
                tmp = np.zeros(K)
                _fold64(xs, K, s * n * dt, dt, float(np.float32(period)), sg[d], tmp,
                        weights=2.0 * np.real(np.conj(xs) * ds))
    P = sx / np.maximum(cx, 1)
    S = (P ** 2).sum(axis=1)
    dS = (2 * P * (sg / np.maximum(cx, 1))).sum(axis=1) if with_grad else None
    return S, dS, plan


CFG = dict(bw=np.float32(4e6), f0=np.float32(400e6), fftpoint=8192, batch=4, period=np.float32(0.0031), nbins=32)


def _signal(n, dm=2.0, seed=7):
    from pymsosm.simulate import pulsar_signal

    return pulsar_signal(n, float(CFG["bw"]), float(CFG["f0"]), dm, float(CFG["period"]), duty=0.05, snr_db=0.0,
                         seed=seed)


@pytest.mark.gpu
def test_checkpoint_resume_is_exact(eng):
    bw, f0, dms, B = np.float32(4e6), np.float32(400e6), [1.0, 2.0, 3.0], 4
    K, period = 32, np.float32(0.0031)

    def make():
        m = eng.MsosmGpuBatch(bw, dms, f0).initialize(0, B, eng.IN_C64, eng.OUT_C64)
        f = eng.FoldGpu(period, bw, B * m.M, K, len(dms))
        m.attach_fold(f)
        return m, f

    rng = np.random.default_rng(31)
    m1, f1 = make()
    n = B * m1.M
    chunks = [(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64) for _ in range(6)]
    outs = []
    for c in chunks:
        m1.filter_block(c)
        o = np.zeros((len(dms), B, m1.M), np.complex64)
        m1.get_output(o)
        m1.synchronize()
        outs.append(o)
    _, s1, c1 = f1.read()

    m2, f2 = make()
    for c in chunks[:2]:
        m2.filter_block(c)
    m2.synchronize()
    st, fst = m2.save_state(), f2.save_state()
    m3, f3 = make()
    m3.load_state(st)
    f3.load_state(fst)
    assert m3.steps == 2
    for k, c in enumerate(chunks[2:], start=2):
        m3.filter_block(c)
        o = np.zeros((len(dms), B, m3.M), np.complex64)
        m3.get_output(o)
        m3.synchronize()
        np.testing.assert_array_equal(o, outs[k])
    _, s3, c3 = f3.read()
    np.testing.assert_array_equal(c3, c1)
    assert rel_l2(s3, s1) < 1e-6
    # a state of another geometry is refused
    other = eng.MsosmGpuBatch(bw, dms, f0).initialize(0, 2, eng.IN_C64, eng.OUT_C64)
    with pytest.raises(eng.MsosmError):
        other.load_state(st)


@pytest.mark.gpu
def test_sharpness_gradient_matches_fp64_and_finite_differences(eng, orc):
    from python_check.dm_autograd import sharpness_and_grad

    dms = [1.7, 2.3]
    # With the segmentation frozen, S(DM) has structure on the scale 1/phi'_max: the
    # band-edge phase moves ~6.5e3 rad per unit DM here, so central differences
    # converge to the derivative only for steps well below 1.5e-4 (measured: 1e-5
    # agrees to ~5e-4 relative; a 1e-3 step is a secant across 6.5 rad and is not).
    h = 1e-5
    x = _signal(6 * 4 * 4096)
    S, dS, _ = sharpness_and_grad(x, CFG["bw"], CFG["f0"], dms, CFG["fftpoint"], CFG["batch"], CFG["period"],
                                  CFG["nbins"])
    S64, dS64, plan = _oracle_sharpness(orc, x, CFG["bw"], CFG["f0"], dms, CFG["fftpoint"], CFG["batch"],
                                        CFG["period"], CFG["nbins"])
    assert np.all(np.abs(S / S64 - 1) < 1e-5)
    assert np.all(np.abs(dS - dS64) <= 1e-3 * np.abs(dS64) + 1e-6 * np.abs(S64))
    # Central differences of the FP64 oracle.  The derivative holds the integer
    # segmentation fixed (it is piecewise constant in DM), so S(DM +- h) uses DM's
    # delay map as well.
    up = np.float32(np.array(dms) + h)
    dn = np.float32(np.array(dms) - h)
    Sp, _, _ = _oracle_sharpness(orc, x, CFG["bw"], CFG["f0"], up, CFG["fftpoint"], CFG["batch"], CFG["period"],
                                 CFG["nbins"], with_grad=False, delays=plan.delays)
    Sm, _, _ = _oracle_sharpness(orc, x, CFG["bw"], CFG["f0"], dn, CFG["fftpoint"], CFG["batch"], CFG["period"],
                                 CFG["nbins"], with_grad=False, delays=plan.delays)
    fd = (Sp - Sm) / (up.astype(np.float64) - dn.astype(np.float64))
    assert np.all(np.abs(dS64 - fd) <= 1e-3 * np.abs(fd) + 1e-6 * np.abs(S64)), (dS64, fd)
    assert np.all(np.abs(dS - fd) <= 2e-3 * np.abs(fd) + 1e-6 * np.abs(S64)), (dS, fd)


@pytest.mark.gpu
def test_autograd_wrapper(eng):
    import torch

    from python_check.dm_autograd import FoldSharpness, sharpness_and_grad

    x = _signal(8 * 4 * 4096, dm=2.0, seed=11)
    dms = torch.tensor([1.6, 2.45], dtype=torch.float64, requires_grad=True)
    S = FoldSharpness.apply(dms, x, CFG)
    w = torch.tensor([0.3, -1.7], dtype=torch.float64)
    (w * S).sum().backward()
    S_ref, dS_ref, _ = sharpness_and_grad(x, CFG["bw"], CFG["f0"], [1.6, 2.45], CFG["fftpoint"], CFG["batch"],
                                          CFG["period"], CFG["nbins"])
    np.testing.assert_allclose(S.detach().numpy(), S_ref, rtol=1e-6)
    np.testing.assert_allclose(dms.grad.numpy(), w.numpy() * dS_ref, rtol=1e-5)
    assert np.isfinite(dS_ref).all() and (dS_ref != 0).all()
