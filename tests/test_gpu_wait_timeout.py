"""Failure detection without a GPU fault: the persistent transform's device-side waits are
bounded.  A wait on a counter that nothing advances runs out after its limit, raises the
error flag and returns; the context stays usable for the next processing call (GPU)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_wait_on_a_counter_nothing_advances_times_out(eng):
    timed_out, ns = eng.selftest_wait(0, 1, 1_000_000)  # 1 ms limit
    assert timed_out
    assert 1_000_000 <= ns < 500_000_000


def test_satisfied_wait_returns_at_once(eng):
    timed_out, ns = eng.selftest_wait(7, 7, 1_000_000)
    assert not timed_out
    assert ns < 1_000_000


def test_limit_is_bounded_by_the_kernel_limit(eng):
    with pytest.raises(eng.MsosmError):
        eng.selftest_wait(0, 1, 3_000_000_000)


def test_context_usable_after_a_timeout(eng, orc):
    eng.selftest_wait(0, 1, 1_000_000)
    bw, f0, dms, B = np.float32(4e6), np.float32(400e6), [1.0, 2.0], 4
    m = eng.MsosmGpuBatch(bw, dms, f0).initialize(1 << 16, B, eng.IN_C64, eng.OUT_C64)
    rng = np.random.default_rng(5)
    ref = orc.Msosm(orc.Plan(bw, f0, dms, 1 << 16, batch=B), B, fp64=True)
    for s in range(2):
        x = (rng.standard_normal(B * m.M) + 1j * rng.standard_normal(B * m.M)).astype(np.complex64)
        m.filter_block(x)
        out = np.zeros((len(dms), B, m.M), np.complex64)
        m.get_output(out)
        m.synchronize()  # reports a timed-out wait of this handle's transform, if any
        r = ref.process(x)
    assert rel_l2(out, r) < 1e-4
