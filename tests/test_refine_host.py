"""Host logic of the DM refinement (pymsosm.refine), on the CPU: the kernel-smoothed
sharpness's analytic first and second derivatives against central differences with
step 1e-3, and the ascent converging on a synthetic comb."""
from __future__ import annotations

import numpy as np

from pymsosm import refine as R


def _comb(rng, centre=123.4, spacing=0.05, k=20):
    c = centre + spacing * np.arange(-k, k + 1)
    S = 1.0 / (1.0 + ((c - 123.37) / 0.3) ** 2) + 1e-3 * rng.standard_normal(c.size)
    return c, S


def test_smoothed_derivatives_match_central_differences():
    rng = np.random.default_rng(1)
    c, S = _comb(rng)
    h = 1e-3
    for d in (122.9, 123.2, 123.41, 123.8):
        f, g, g2 = R.smoothed_sharpness(d, c, S, 0.1)
        fp, gp, _ = R.smoothed_sharpness(d + h, c, S, 0.1)
        fm, gm, _ = R.smoothed_sharpness(d - h, c, S, 0.1)
        assert abs(g - (fp - fm) / (2 * h)) <= 1e-3 * abs(g) + 1e-9
        assert abs(g2 - (gp - gm) / (2 * h)) <= 1e-3 * abs(g2) + 1e-9


def test_ascent_on_a_synthetic_comb(monkeypatch):
    rng = np.random.default_rng(2)

    def fake(x, bw, f0, comb, period, nbins, fftpoint=0):
        return 1.0 / (1.0 + ((np.asarray(comb) - 57.25) / 0.3) ** 2) + 1e-4 * rng.standard_normal(len(comb))

    monkeypatch.setattr(R, "comb_sharpness", fake)
    for guess in (56.75, 57.75):
        est, tr = R.refine_dm(None, 1.0, 1.0, guess, 1.0)
        assert len(tr.dm) == 20
        assert abs(est - 57.25) < 0.01
