"""The numpy model of the GPU simulator, on the CPU: its counter-based generator
against the published Philox-4x32-10 known-answer vectors (Random123's kat_vectors),
its normals' moments, and its dispersion response against the engine's own
plan (the FP64 causal response the simulator applies)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_sim as osim

# (counter words, key words, expected output words), Philox-4x32-10
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(ctr, key, want):
    out = osim.philox_rounds(*[np.array([c], np.uint64) for c in ctr], *key)
    assert tuple(int(w[0]) for w in out) == want


def test_normal_pairs_moments():
    g = osim.normal_pairs(np.arange(1 << 20, dtype=np.uint64), 0, 7)
    for q in (g.real, g.imag):
        assert abs(q.mean()) < 5e-3 and abs(q.std() - 1) < 5e-3
    assert abs(np.mean(g.real * g.imag)) < 5e-3


@pytest.mark.parametrize("bw,f0,dm", [(16e6, 1392e6, 50.0), (8e6, 1000e6, 20.0), (64e6, 1368e6, 123.4)])
def test_dispersion_taps_hold_the_chirp_energy(bw, f0, dm):
    """The Nd + 1 causal taps keep nearly all of the chirp response's unit energy
    (the rest lies outside the smear window the reference's construction keeps)."""
    nd = osim.smear(bw, dm, f0)
    taps = osim.dispersion_taps(bw, f0, dm, nd)
    e = float(np.sum(np.abs(taps) ** 2))
    assert 0.99 < e <= 1.0 + 1e-9


def test_smear_matches_engine_plan(eng):
    bw, f0 = np.float32(64e6), np.float32(1368e6)
    for dm in (0.0, 50.0, 123.4, 200.0):
        nd_osm, _ = eng.osm_plan(bw, np.float32(dm), f0)
        assert osim.smear(bw, dm, f0) == nd_osm
