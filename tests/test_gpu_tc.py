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
