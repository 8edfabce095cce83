"""Host-side pieces of bench.py on CPU: the workloads' DM grids and synthetic baseband."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def test_many_dm_grid_is_the_linear_grid():
    g = bench.dm_grid(bench.WORKLOADS["many_dm_512"])
    assert g.dtype == np.float32 and len(g) == 512
    assert g[0] == 0.0 and g[-1] == np.float32(200.0) and np.all(np.diff(g) > 0)


def test_two_pol_grid_is_sorted_log_uniform_and_shards_evenly():
    w = bench.WORKLOADS["two_pol_1024"]
    g = bench.dm_grid(w)
    assert len(g) == 1024 and np.all(np.diff(g) >= 0)
    assert g[0] >= 1.0 and g[-1] <= 1000.0
    # log-uniform: about half the trials below the geometric midpoint
    assert 400 < int(np.sum(g < np.sqrt(1000.0))) < 624
    shards = [bench.dm_grid(w, r, 2) for r in range(2)]
    assert [len(s) for s in shards] == [1024, 1024]  # each rank: a full share of a 2048 grid
    merged = np.sort(np.concatenate(shards))
    assert np.all(np.diff(merged) >= 0) and np.all(np.diff(shards[0]) >= 0)


def test_int8_baseband_is_clipped_gaussian_and_seeded():
    x = bench.int8_baseband(1 << 16, 20.0, 7)
    assert x.dtype == np.int8 and x.size == 2 << 16
    assert x.min() >= -127 and x.max() <= 127
    assert abs(float(np.std(x.astype(np.float64))) - 20.0) < 0.5
    np.testing.assert_array_equal(x, bench.int8_baseband(1 << 16, 20.0, 7))


def test_workload_config_is_the_same_object_for_both_arms():
    """Both arms print workload_config(); its sizes follow the workload, and only the
    workloads whose step fits in L2 are timed with L2 overwritten between steps."""
    import types

    for name, w in bench.WORKLOADS.items():
        if "n_sources" in w:
            continue
        args = types.SimpleNamespace(workload=name, precision="fp32")
        c = bench.workload_config(args, dict(w), 2)
        assert c == bench.workload_config(args, dict(w), 2)
        assert c["workload"] == name and c["fft_size"] == w["fftpoint"] and c["M"] == w["fftpoint"] // 2
        assert c["dm_trials_per_gpu"] == w["n_dms"] and c["batch"] == w["batch"]
        assert c["parallelism"] == "dm-shard x2"
        assert ("L2 flushed" in c["l2"]) == bench.fits_in_l2(w)
    assert not bench.fits_in_l2(bench.WORKLOADS["many_dm_512"])
    assert not bench.fits_in_l2(bench.WORKLOADS["two_pol_1024"])
    assert bench.fits_in_l2(bench.WORKLOADS["single_dm_50"])
