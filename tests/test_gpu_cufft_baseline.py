"""The cuFFT restatement of the reference's GPU design (the baseline bench.py times beside
the engine) folds the same profiles as the engine and the FP64 oracle (GPU)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

LIB = Path(__file__).resolve().parents[1] / "baseline" / "cufft_pipeline" / "lib" / "libmsosm_cufft_pipeline.so"


def _lib():
    if not LIB.exists():
        pytest.fail(f"{LIB} is missing: run __graft_entry__.build()")
    L = C.CDLL(str(LIB))
    L.mcp_create.argtypes = [C.c_int] * 6 + [C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]
    L.mcp_process.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcp_read.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcp_destroy.argtypes = [C.c_void_p]
    return L


def test_cufft_design_folds_like_the_engine(eng, orc):
    import torch

    bw, f0 = np.float32(16e6), np.float32(1392e6)
    dms = np.array([10.0, 25.0, 40.0, 50.0], np.float32)
    B, K, period, calls = 4, 128, np.float32(0.0071), 4
    proc = eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 16, B, eng.IN_C64, eng.OUT_C64)
    fold = eng.FoldGpu(period, bw, B * proc.M, K, len(dms))
    proc.attach_fold(fold)
    F, M = proc.fftpoint, proc.M
    rng = np.random.default_rng(11)
    x = (rng.standard_normal(calls * B * M) + 1j * rng.standard_normal(calls * B * M)).astype(np.complex64)
    dev = torch.device("cuda:0")
    dx = torch.from_numpy(x.view(np.float32)).to(dev)
    H = torch.stack([torch.from_numpy(proc.response(i)) for i in range(len(dms))]).to(dev)
    dl = torch.stack([torch.from_numpy(proc.delay_points(i).astype(np.uint16).view(np.int16))
                      for i in range(len(dms))]).to(dev)
    L = _lib()
    h = C.c_void_p()
    assert L.mcp_create(16, B, len(dms), proc.ring_blocks, 2, K, period, bw, H.data_ptr(), dl.data_ptr(),
                        C.byref(h)) == 0
    try:
        series = []
        for c in range(calls):
            proc.filter_block(dx[c * 2 * B * M:(c + 1) * 2 * B * M])
            o = np.zeros((len(dms), B, M), np.complex64)
            proc.get_output(o)
            proc.synchronize()
            series.append(o)
            assert L.mcp_process(h, C.c_void_p(dx.data_ptr() + c * B * M * 8), None) == 0
        sums = np.zeros((len(dms), K))
        cnts = np.zeros((len(dms), K), np.uint64)
        assert L.mcp_read(h, sums.ctypes.data, cnts.ctypes.data) == 0
    finally:
        L.mcp_destroy(h)
    _, esums, ecnts = fold.read()
    assert np.abs(cnts.astype(np.int64) - ecnts.astype(np.int64)).sum() <= 2 * len(dms)
    assert rel_l2(sums, esums) < 1e-4
    # and both fold the FP64 oracle's series of the first trial
    plan = orc.Plan(bw, f0, dms[:1], F, batch=B)
    om = orc.Msosm(plan, B, fp64=True)
    s_ = np.zeros(K)
    c_ = np.zeros(K, np.uint64)
    dt = 1.0 / float(bw)
    for c in range(calls):
        r = om.process(x[c * B * M:(c + 1) * B * M])[0].reshape(-1)
        orc.fold(np.abs(r) ** 2, K, c * B * M * dt, dt, float(period), s_, c_)
    assert rel_l2(sums[0], s_) < 1e-4
