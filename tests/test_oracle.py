"""The oracle pinned against the reference (CPU only).

The golden fixtures in tests/golden were produced by the reference's own
planning sources (dedispersion/msosm/msosm_prepare.cpp, overlap_save/osm_prepare.cpp)
compiled unmodified; see tests/golden/make_golden.py.  The streaming restatement
is checked against an independent numpy FP64 model of the same recurrence.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import expand_runs, rel_l2


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128, 256, 1024, 4096])
def test_fft_matches_numpy(orc, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    assert rel_l2(orc.fft(x, -1), np.fft.fft(x)) < 1e-13
    assert rel_l2(orc.fft(x, +1), np.fft.ifft(x) * n) < 1e-13
    assert rel_l2(orc.fft(x, -1, fp64=False), np.fft.fft(x)) < 2e-6


def _case_plan(orc, c, with_response=False):
    return orc.Plan(c["bw"], c["f0"], c["dms"], c["fftpoint"], batch=4, with_response=with_response)


def test_plan_cases_match_reference(orc, golden_plans):
    """Nd, M_min, M, delaycount and every delay map: bit-exact vs the reference build."""
    for name, c in golden_plans.items():
        p = _case_plan(orc, c)
        assert p.nd.tolist() == c["nd"], name
        assert p.M_min == c["M_min"], name
        assert p.M == c["M"], name
        assert p.dc.tolist() == c["dc"], name
        assert p.delaycount == c["delaycount"], name
        for i, runs in enumerate(c["delay_runs"]):
            if runs is None:  # DM 0: the reference leaves the map uninitialised
                assert c["dc"][i] == 0
                assert not p.delays[i].any()
                continue
            np.testing.assert_array_equal(p.delays[i], expand_runs(runs, p.F), err_msg=f"{name} DM#{i}")


def test_response_matches_reference(orc, golden_plans, golden_arrays):
    for name, c in golden_plans.items():
        M = c["M"]
        if f"{name}__H" in golden_arrays:
            Href = golden_arrays[f"{name}__H"]
            for i, dm in enumerate(c["dms"]):
                H = orc.response(c["bw"], c["f0"], dm, M)
                assert rel_l2(H, Href[i]) < 2e-6, (name, i)
        else:
            if M > (1 << 17):
                continue  # the 2^20-point FP64 responses are covered by the product tests
            idx = golden_arrays[f"{name}__Hidx"]
            for k, i in enumerate(golden_arrays[f"{name}__Hsel"]):
                H = orc.response(c["bw"], c["f0"], c["dms"][i], M)
                assert rel_l2(H[idx], golden_arrays[f"{name}__Hsample"][k]) < 5e-6, (name, i)
                assert abs(np.linalg.norm(H) / golden_arrays[f"{name}__Hnorm"][i] - 1) < 1e-6


def test_osm_plan_matches_reference(orc, golden_osm, golden_arrays):
    for name, c in golden_osm.items():
        nd = orc.osm_nd(c["bw"], c["dm"], c["f0"])
        assert nd == c["nd"], name
        mmin = orc.osm_min_order(nd)
        assert mmin == c["M_min"], name
        M = max(c["fftpoint"] // 2, mmin) if c["fftpoint"] else mmin
        assert M == c["M"], name
        if M <= (1 << 16):
            H = orc.response(c["bw"], c["f0"], c["dm"], M)
            idx = golden_arrays[f"{name}__Hidx"]
            assert rel_l2(H[idx], golden_arrays[f"{name}__Hsample"]) < 5e-6


def test_response_even_bins_are_the_chirp(orc):
    """H[2k] equals the FFT-order chirp exactly (FFT_M inverts IFFT_M)."""
    bw, f0, dm, M = np.float32(4e6), np.float32(400e6), 3.0, 1024
    H = orc.response(bw, f0, dm, M)
    j = np.arange(M)
    w = 2 * np.pi * float(bw) * j / M
    w0 = 2 * np.pi * float(f0)
    phase = 4 * np.pi ** 2 * 4.15e15 * float(np.float32(dm)) * w * w / ((w + w0) * w0 * w0)
    c = np.empty(M, np.complex128)
    dst = np.where(j < M // 2, M // 2 + j, j - M // 2)
    c[dst] = np.exp(-1j * phase)
    assert np.abs(H[0::2] - c).max() < 1e-9


def _numpy_msosm(x, plan, B, steps):
    """Independent FP64 model: output block g of DM d reads spectrum g - delay[n]."""
    M, F = plan.M, plan.F
    total = B * steps
    stream = np.concatenate([np.zeros(M, np.complex128), x.astype(np.complex128)])
    spec = np.stack([np.fft.fft(stream[g * M:g * M + F]) for g in range(total)])
    out = np.zeros((len(plan.dms), total, M), np.complex128)
    n = np.arange(F)
    for d in range(len(plan.dms)):
        for g in range(total):
            src = g - plan.delays[d]
            xs = np.where(src >= 0, spec[np.clip(src, 0, None), n], 0)
            y = np.fft.ifft(xs * plan.H[d]) * F
            out[d, g] = y[M:] / F
    return out


def test_streaming_matches_numpy_model(orc):
    """Ring, tail hand-over and gather of the restated stream, over several ring wraps."""
    plan = orc.Plan(np.float32(4e6), np.float32(400e6), [1.0, 2.0, 3.0], 0, batch=2)
    B, steps = 2, 7
    rng = np.random.default_rng(1)
    x = rng.standard_normal(B * plan.M * steps) + 1j * rng.standard_normal(B * plan.M * steps)
    ref = _numpy_msosm(x, plan, B, steps)
    m = orc.Msosm(plan, B, fp64=True, nthreads=2)
    assert m.fbs == plan.fbs
    got = np.concatenate([m.process(x[s * B * plan.M:(s + 1) * B * plan.M]) for s in range(steps)], axis=1)
    assert rel_l2(got, ref) < 1e-12


def test_dm0_is_identity(orc):
    plan = orc.Plan(np.float32(4e6), np.float32(400e6), [0.0], 2048, batch=2)
    assert plan.delaycount == 0 and not plan.delays.any()
    m = orc.Msosm(plan, 2, fp64=True, nthreads=1)
    rng = np.random.default_rng(2)
    for _ in range(3):
        x = rng.standard_normal(2 * plan.M) + 1j * rng.standard_normal(2 * plan.M)
        y = m.process(x)
        assert np.abs(y.reshape(-1) - x).max() < 1e-12


def test_fp32_port_matches_fp64(orc):
    plan = orc.Plan(np.float32(8e6), np.float32(600e6), [0.5, 2.5, 8.0], 0, batch=4)
    rng = np.random.default_rng(3)
    a = orc.Msosm(plan, 4, fp64=True, nthreads=2)
    b = orc.Msosm(plan, 4, fp64=False, nthreads=2)
    for _ in range(3):
        x = (rng.standard_normal(4 * plan.M) + 1j * rng.standard_normal(4 * plan.M)).astype(np.complex64)
        assert rel_l2(b.process(x), a.process(x)) < 1e-5


def test_u16_decode_known_answers(orc):
    v = np.array([0, 32768, 1, 65535, (1 << 16) | 32768, (32768 << 16) | 0], np.uint32)
    got = orc.decode_u16(v)
    exp = np.array([0, 0, -32767, 32767, 0 + 1j * (1 - 32768), 0], np.complex64)
    np.testing.assert_array_equal(got, exp)


def test_u16_encode_known_answers(orc):
    # discardSamplesToUint16: rn(v + 32768*(v != 0)), packed (y << 16) | x
    vals = np.array([0.0, 0.4, -0.6, 1.5, 2.5, -40000.0, 32767.6], np.float32)
    x = vals.astype(np.complex64)
    got = orc.encode_u16(x)
    exp_x = [0, 32768, 32767, 32770, 32770, 0, 65536]  # 65535.6 rounds to 65536 and spills into y
    exp = [(e & 0xFFFFFFFF) for e in exp_x]
    np.testing.assert_array_equal(got, np.array(exp, np.uint32))


def test_i8_decode(orc):
    iq = np.array([0, 0, -128, 127, 5, -7], np.int8)
    np.testing.assert_array_equal(orc.decode_i8(iq), np.array([0, -128 + 127j, 5 - 7j], np.complex64))


def test_fold_known_answer(orc):
    # period 1 s, dt 0.25 s, 4 bins: samples land in bins 0,1,2,3,0,1,...
    inten = np.array([1, 2, 3, 4, 5, 0, 7, 8], np.float32)
    s, c = orc.fold(inten, 4, 0.0, 0.25, 1.0)
    np.testing.assert_allclose(s, [6, 2, 10, 12])
    np.testing.assert_array_equal(c, [2, 1, 2, 2])  # the zero sample is skipped
    np.testing.assert_allclose(orc.fold_finalize(s, c), [3, 2, 5, 6])


def test_build_segments_matches_the_reference(orc, golden_plans):
    """The oracle's build_segments restatement against the reference's own
    MSOSM_GPU_BATCH::build_segments (msosm_gpu_batch.cpp:262-295) run on the same
    delay maps (tests/golden/segment_cases.json): same triples, every DM of every case."""
    import hashlib
    import json

    from conftest import GOLDEN, expand_runs

    ref = json.loads((GOLDEN / "segment_cases.json").read_text())
    checked = 0
    for name, per in ref.items():
        case = golden_plans[name]
        F = 2 * case["M"]
        for i, e in enumerate(per):
            if e is None:
                assert case["delay_runs"][i] is None
                continue
            st, ln, gr = orc.build_segments(expand_runs(case["delay_runs"][i], F))
            tri = np.stack([st, ln, gr], axis=1).astype("<i4")
            assert len(tri) == e["count"], (name, i)
            assert hashlib.sha256(tri.tobytes()).hexdigest() == e["sha256"], (name, i)
            if "triples" in e:
                assert tri.tolist() == e["triples"]
            checked += 1
    assert checked == 591  # all DMs but the many-DM grid's DM 0
