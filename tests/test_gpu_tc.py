"""Tensor-core (tcgen05) pieces of the split-precision transform, through the C ABI."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """float -> bfloat16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def _bf16_value(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("bf16", [True, False])
@pytest.mark.parametrize("n,row0", [(64, 0), (32, 32), (32, 0)])
def test_umma_operand_layout(eng, bf16, n, row0):
    rng = np.random.default_rng(7 + n + row0 + int(bf16))
    a = rng.standard_normal((128, 64))
    b = rng.standard_normal((64, 64))
    if bf16:
        A, B = _to_bf16_bits(a), _to_bf16_bits(b)
        av, bv = _bf16_value(A), _bf16_value(B)
    else:
        A, B = a.astype(np.float16).view(np.uint16), b.astype(np.float16).view(np.uint16)
        av, bv = A.view(np.float16).astype(np.float64), B.view(np.float16).astype(np.float64)
    D = eng.selftest_umma(A, B, n=n, b_row0=row0, bf16=bf16)
    ref = av @ bv[row0:row0 + n].T
    err = np.abs(D - ref).max()
    assert err < 1e-4 * np.abs(ref).max(), err


def _oracle_windows(orc, bw, f0, dms, F, B):
    plan = orc.Plan(bw, f0, dms, F, batch=B)
    return orc.Msosm(plan, B, fp64=True)


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_split_precision_matches_fp64_oracle(eng, orc, prec):
    """A few DM trials at F = 2^18 through the tensor-core transform, series against the
    FP64 oracle after the ring warm-up, next to the FP32 register transform."""
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    dms = np.array([0.0, 20.0, 57.5, 123.4, 200.0], np.float32)
    F, B, calls = 1 << 18, 4, 3
    code = {"bf16": eng.PREC_BF16X3, "fp16": eng.PREC_FP16X3}[prec]
    m_tc = eng.MsosmGpuBatch(bw, dms, f0).initialize(F, B, eng.IN_C64, eng.OUT_C64).set_precision(code)
    m_32 = eng.MsosmGpuBatch(bw, dms, f0).initialize(F, B, eng.IN_C64, eng.OUT_C64)
    assert m_tc.precision == code and m_32.precision == eng.PREC_FP32
    om = _oracle_windows(orc, bw, f0, dms, F, B)
    dc = m_tc.delaycounts()
    rng = np.random.default_rng(31)
    out_tc = np.zeros((len(dms), B, m_tc.M), np.complex64)
    out_32 = np.zeros_like(out_tc)
    e_tc = np.zeros(len(dms))
    e_32 = np.zeros(len(dms))
    den = np.zeros(len(dms))
    for s in range(calls):
        # loud input: spectra near 2^13 per bin, so the FP16 operand scaling is exercised
        x = (40 * (rng.standard_normal(B * m_tc.M) + 1j * rng.standard_normal(B * m_tc.M))).astype(np.complex64)
        m_tc.filter_block(x)
        m_32.filter_block(x)
        m_tc.get_output(out_tc)
        m_32.get_output(out_32)
        m_tc.synchronize()
        m_32.synchronize()
        r = om.process(x)
        for d in range(len(dms)):
            w0 = max(0, dc[d] + 1 - s * B)
            if w0 >= B:
                continue
            rr = r[d, w0:]
            den[d] += float(np.vdot(rr, rr).real)
            dt = out_tc[d, w0:].astype(np.complex128) - rr
            d3 = out_32[d, w0:].astype(np.complex128) - rr
            e_tc[d] += float(np.vdot(dt, dt).real)
            e_32[d] += float(np.vdot(d3, d3).real)
    ok = den > 0
    rel_tc = np.sqrt(e_tc[ok] / den[ok])
    rel_32 = np.sqrt(e_32[ok] / den[ok])
    print(f"{prec}: per-trial rel-L2 vs FP64 {np.array2string(rel_tc, precision=2)}; "
          f"FP32 path {np.array2string(rel_32, precision=2)}")
    assert ok.sum() >= 3
    assert rel_tc.max() < 1e-4


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_split_precision_fused_fold(eng, prec):
    """Fold-only processing through the tensor-core transform gives the FP32 path's
    folded profiles (same counts, profiles within 1e-4) and the same peak bin."""
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    dms = np.linspace(100.0, 140.0, 9).astype(np.float32)
    F, B, K, calls = 1 << 18, 8, 512, 3
    code = {"bf16": eng.PREC_BF16X3, "fp16": eng.PREC_FP16X3}[prec]
    from pymsosm import simulate

    profs = []
    for p in (eng.PREC_FP32, code):
        m = eng.MsosmGpuBatch(bw, dms, f0).initialize(F, B, eng.IN_C64, eng.OUT_NONE).set_precision(p)
        fold = eng.FoldGpu(np.float32(0.033), bw, B * m.M, K, len(dms))
        m.attach_fold(fold)
        n = B * m.M * calls
        x = simulate.pulsar_signal(n, float(bw), float(f0), 123.4, 0.033, snr_db=-10.0, seed=3)
        for s in range(calls):
            m.filter_block(np.ascontiguousarray(x[s * B * m.M:(s + 1) * B * m.M]))
        m.synchronize()
        folded, _, cnt = fold.read()
        profs.append((folded.copy(), cnt.copy()))
    (f32, c32), (ftc, ctc) = profs
    assert np.array_equal(c32, ctc)
    rel = np.linalg.norm(ftc - f32) / np.linalg.norm(f32)
    print(f"{prec}: folded profiles vs FP32 path rel-L2 {rel:.2e}")
    assert rel < 1e-4
    best = int(np.argmax(f32.max(axis=1) - f32.mean(axis=1)))
    assert int(np.argmax(ftc[best])) == int(np.argmax(f32[best]))
