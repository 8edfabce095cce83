"""DM refinement by gradient ascent on a smoothed folded-profile sharpness.

Sharpness of a DM trial d: S(d) = sum_k (P_k - mean P)^2 over the folded intensity
profile P (mean |x|^2 per phase bin, mean-subtracted so that trials with different
noise levels compare).  S(d) of coherently dedispersed baseband is not smooth on small
DM scales: the intensity pattern of noise-like emission and noise decorrelates once the
extra group delay across the band reaches about one sample (about 1e-4 DM at 16-64 MHz),
and the multi-segment approximation adds block-boundary terms whose phase turns with
the chirp's DM derivative (1e3-1e5 rad per DM unit at the band edge).  Its exact
derivative (msosm_use_response_derivative + msosm_fold_accumulate_cross) is dominated
by that fine structure and does not predict the change of S over 1e-3 DM.

The refinement therefore ascends a kernel-smoothed sharpness on a fixed comb of trial
DMs c_q evaluated in ONE many-DM pass of the engine (all trials share the forward
transform; the fused fold gives every trial's profile):

    S~(d) = sum_q w_q(d) S(c_q) / sum_q w_q(d),   w_q(d) = exp(-(d - c_q)^2 / (2 sigma^2))

S~ is smooth in d, and its derivative, with w'_q = -(d - c_q)/sigma^2 w_q,

    dS~/dd = (sum_q w'_q S(c_q) - S~ sum_q w'_q) / sum_q w_q

is exact and agrees with central differences at any step.  Coarse to fine: a wide comb
(spacing 0.05 DM, +-1 DM, sigma 0.1) for the first half of the steps, then a narrow comb
(spacing 0.005 DM, +-0.1 DM, sigma 0.01) around the estimate for the rest.  A step is
Newton's where S~ is concave, else one sigma uphill, and never leaves the comb.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import IN_C64, OUT_NONE, FoldGpu, MsosmGpuBatch


@dataclass
class Stage:
    spacing: float
    half_width: float
    sigma: float
    steps: int


DEFAULT_STAGES = (Stage(0.05, 1.0, 0.1, 10), Stage(0.005, 0.1, 0.01, 10))


def comb_sharpness(x: np.ndarray, bw: float, f0: float, comb: np.ndarray, period: float, nbins: int,
                   fftpoint: int = 0) -> np.ndarray:
    """S(c_q) of every comb DM for baseband x (complex64, host or device), one engine pass.

    The batch is chosen so that one step covers the largest trial's ring warm-up
    ((delaycount + 1) * M samples); the fold is attached from the second step on."""
    comb = np.ascontiguousarray(np.asarray(comb, np.float32))
    probe = MsosmGpuBatch(np.float32(bw), comb, np.float32(f0)).initialize(fftpoint, 1, IN_C64, OUT_NONE)
    B = int(probe.delaycount) + 1
    M = int(probe.M)
    del probe
    n = B * M
    steps = len(x) // n
    if steps < 2:
        raise ValueError(f"source of {len(x)} samples is shorter than two steps of {n}")
    m = MsosmGpuBatch(np.float32(bw), comb, np.float32(f0)).initialize(fftpoint, B, IN_C64, OUT_NONE)
    fold = FoldGpu(np.float32(period), np.float32(bw), n, nbins, len(comb))
    for s in range(steps):
        if s == 1:
            m.attach_fold(fold)
        m.filter_block(np.ascontiguousarray(x[s * n:(s + 1) * n]) if isinstance(x, np.ndarray) else x[s * n:(s + 1) * n])
    m.synchronize()
    prof, _, _ = fold.read()
    p = prof.astype(np.float64)
    p -= p.mean(axis=1, keepdims=True)
    return (p * p).sum(axis=1)


def smoothed_sharpness(d: float, comb: np.ndarray, S: np.ndarray, sigma: float) -> tuple[float, float, float]:
    """(S~(d), dS~/dd, d2S~/dd2) of the kernel-smoothed sharpness."""
    u = (d - np.asarray(comb, np.float64)) / sigma
    w = np.exp(-0.5 * u * u)
    dw = -u / sigma * w
    d2w = (u * u - 1.0) / (sigma * sigma) * w
    W, W1, W2 = w.sum(), dw.sum(), d2w.sum()
    N0, N1, N2 = (w * S).sum(), (dw * S).sum(), (d2w * S).sum()
    f = N0 / W
    f1 = (N1 - f * W1) / W
    f2 = (N2 - 2.0 * f1 * W1 - f * W2) / W
    return float(f), float(f1), float(f2)


@dataclass
class Trace:
    dm: list = field(default_factory=list)
    value: list = field(default_factory=list)
    grad: list = field(default_factory=list)


def refine_dm(x: np.ndarray, bw: float, f0: float, dm0: float, period: float, nbins: int = 256,
              stages=DEFAULT_STAGES, fftpoint: int = 0) -> tuple[float, Trace]:
    """Refine one source's DM from the guess dm0; returns (estimate, per-step trace)."""
    d = float(dm0)
    tr = Trace()
    for st in stages:
        k = int(round(st.half_width / st.spacing))
        comb = d + st.spacing * np.arange(-k, k + 1)
        comb = comb[comb >= 0.0]
        S = comb_sharpness(x, bw, f0, comb, period, nbins, fftpoint)
        lo, hi = float(comb[0]), float(comb[-1])
        for _ in range(st.steps):
            f, g, h = smoothed_sharpness(d, comb, S, st.sigma)
            tr.dm.append(d)
            tr.value.append(f)
            tr.grad.append(g)
            step = -g / h if h < 0 else np.sign(g) * st.sigma
            step = float(np.clip(step, -st.sigma, st.sigma))
            d = float(np.clip(d + step, lo, hi))
    return d, tr
