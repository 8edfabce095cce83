"""msosm_osm_filter_noalloc: overlap-save filtering that allocates no device memory.

The entry point exists for callers that cannot allocate device memory while
filtering -- real-time loops that allocate everything up front (cudaMalloc and
cudaFree synchronise the device and can miss a buffer deadline) and plug-ins
whose host application owns the GPU's memory budget.  Its intermediates live in
a fixed file-scope device array, so this test checks, through the C ABI, that
consecutive calls with alternating FFT sizes (the smallest, a middle one, and one
that fills the array) give the same output as the allocating processor
(osm_create + msosm_process) on the same windows, within the parity tolerance,
and that requests larger than the array are refused.

This file is collected last on purpose; it must pass both alone in a fresh
process and after the rest of the suite.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4
UNSUPPORTED = 5


def _noalloc(eng):
    L = eng.lib()
    f = L.msosm_osm_filter_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _reference_windows(m, x, count):
    """The allocating processor's output for windows over x ((count+1)*M samples)."""
    M = m.M
    lead = np.zeros(count * M, np.complex64)
    lead[-M:] = x[:M]  # leaves x[:M] as the history of the next call
    m.filter_block(lead)
    m.filter_block(np.ascontiguousarray(x[M:]))
    out = np.zeros((1, count, M), np.complex64)
    m.get_output(out)
    m.synchronize()
    return out.reshape(-1)


# (fftpoint, windows per call, DM): the smallest geometry (N1 = N2 = 16), a
# mid-size one, and one request that fills the array (count * fftpoint = 2^20)
# with the 1024-point sub-transforms
CASES = [(1 << 8, 64, 0.02), (1 << 18, 4, 0.5), (1 << 20, 1, 0.5)]


def test_noalloc_matches_processor_alternating_sizes(eng):
    import torch

    f = _noalloc(eng)
    bw, f0 = np.float32(4e6), np.float32(400e6)
    procs = []
    for F, count, dm in CASES:
        m = eng.OsmGpuBatch(bw, dm, f0).initialize(F, count, eng.IN_C64, eng.OUT_C64)
        assert m.fftpoint == F
        H = torch.from_numpy(m.response(0).view(np.float32)).cuda()
        procs.append((F, count, m, H))
    rng = np.random.default_rng(2024)
    # two rounds over the sizes: every call follows a call with another fftpoint,
    # so state left in the array by a different geometry would show
    for rnd in range(2):
        for F, count, m, H in procs:
            M = m.M
            x = (rng.standard_normal((count + 1) * M) + 1j * rng.standard_normal((count + 1) * M)).astype(
                np.complex64)
            dx = torch.from_numpy(x.view(np.float32)).cuda()
            dout = torch.full((2 * count * M,), float("nan"), dtype=torch.float32, device="cuda")
            stream = torch.cuda.current_stream().cuda_stream
            rc = f(dx.data_ptr(), H.data_ptr(), F, count, dout.data_ptr(), stream)
            assert rc == 0
            torch.cuda.synchronize()
            got = dout.cpu().numpy().view(np.complex64)
            ref = _reference_windows(m, x, count)
            assert np.isfinite(got).all()
            err = rel_l2(got, ref)
            assert err < TOL, (rnd, F, count, err)


def test_noalloc_refuses_oversized_requests(eng):
    import torch

    f = _noalloc(eng)
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    p = buf.data_ptr()
    assert f(p, p, 1 << 20, 2, p, None) == UNSUPPORTED  # count*fftpoint above 2^20
    assert f(p, p, 1 << 21, 1, p, None) == UNSUPPORTED  # fftpoint above 2^20
    assert f(p, p, 3000, 1, p, None) == UNSUPPORTED  # not a power of two
