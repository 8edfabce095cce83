"""Test-only harness: folded-profile sharpness and its DM derivative as a
torch.autograd.Function, over the engine's C ABI.

Sharpness of DM trial d: S_d = sum_k P_{d,k}^2, P_{d,k} = mean |x|^2 in phase bin k.
With the segmentation held fixed, x depends on DM only through the response, so
dx/dDM is the same pipeline run with dH/dDM (msosm_use_response_derivative), and
dS/dDM = sum_k 2 P_k (sum 2 Re(conj(x) dx) / n_k)  (msosm_fold_accumulate_cross).
Nothing is stored between passes: each evaluation recomputes the segments from
the baseband.
"""
from __future__ import annotations

import numpy as np
import torch

import pymsosm as eng


def sharpness_and_grad(x: np.ndarray, bw, f0, dms, fftpoint, batch, period, nbins):
    """(S[D], dS/dDM[D], P[D][K]) for complex64 baseband x through the engine."""
    dms = np.ascontiguousarray(np.asarray(dms, np.float32))
    hx = eng.MsosmGpuBatch(bw, dms, f0).initialize(fftpoint, batch, eng.IN_C64, eng.OUT_C64)
    hd = eng.MsosmGpuBatch(bw, dms, f0).initialize(fftpoint, batch, eng.IN_C64, eng.OUT_C64)
    hd.use_response_derivative()
    n = hx.batch * hx.M
    fx = eng.FoldGpu(np.float32(period), np.float32(bw), n, nbins, len(dms))
    fg = eng.FoldGpu(np.float32(period), np.float32(bw), n, nbins, len(dms))
    for s in range(len(x) // n):
        chunk = np.ascontiguousarray(x[s * n:(s + 1) * n])
        hx.filter_block(chunk)
        hd.filter_block(chunk)
        fx.accumulate(hx.get_output_pointer())
        fg.accumulate_cross(hx.get_output_pointer(), hd.get_output_pointer())
    hx.synchronize()
    _, sx, cx = fx.read()
    _, sg, cg = fg.read()
    assert np.array_equal(cx, cg)
    cnt = np.maximum(cx.astype(np.float64), 1.0)
    P = sx / cnt
    dP = sg / cnt
    S = (P ** 2).sum(axis=1)
    dS = (2.0 * P * dP).sum(axis=1)
    return S, dS, P


class FoldSharpness(torch.autograd.Function):
    """S(dms) with d S / d dms from the engine's derivative pass."""

    @staticmethod
    def forward(ctx, dms: torch.Tensor, x: np.ndarray, cfg: dict):
        S, dS, _ = sharpness_and_grad(x, cfg["bw"], cfg["f0"], dms.detach().cpu().numpy(), cfg["fftpoint"],
                                      cfg["batch"], cfg["period"], cfg["nbins"])
        ctx.save_for_backward(torch.from_numpy(dS).to(dms.dtype))
        return torch.from_numpy(S).to(dms.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (dS,) = ctx.saved_tensors
        return grad_out * dS, None, None
