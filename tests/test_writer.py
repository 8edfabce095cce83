"""Per-DM output files (the data_save front end) through the C ABI."""
from __future__ import annotations

import os

import numpy as np
import pytest


@pytest.mark.parametrize("dms,prefix,names", [
    ([75.0], "", ["DM75.00.dat"]),  # integers print with 2 decimals
    ([1.5, 2.25], "sim", ["sim_DM1.50.dat", "sim_DM2.25.dat"]),  # decimals of the first two DMs
    ([0.0, 0.5, 1.0], "", ["DM0.0.dat", "DM0.5.dat", "DM1.0.dat"]),  # DM 0 needs none
])
def test_file_names_follow_the_reference(eng, tmp_path, dms, prefix, names):
    w = eng.Writer(tmp_path, prefix, dms, 4096)
    assert [os.path.basename(n) for n in w.filenames()] == names
    w.close()


def test_blocks_land_at_step_offsets(eng, tmp_path):
    rng = np.random.default_rng(3)
    D, per = 3, 8192
    w = eng.Writer(tmp_path, "t", [1.0, 2.0, 3.0], per, slots=2)
    blocks = [rng.integers(0, 2 ** 32, (D, per // 4), dtype=np.uint32) for _ in range(7)]
    for b in blocks:
        w.write(b)
    w.join()
    for d, name in enumerate(w.filenames()):
        got = np.fromfile(name, np.uint32)
        np.testing.assert_array_equal(got, np.concatenate([b[d] for b in blocks]))
    w.close()


def test_reader_decodes_offset_binary(eng, tmp_path):
    p = tmp_path / "x.dat"
    np.array([0, 32768, (32769 << 16) | 32767, (1 << 16) | 65535], np.uint32).tofile(p)
    np.testing.assert_array_equal(eng.read_dat(p), np.array([0, 0, -1 + 1j, 32767 - 32767j], np.complex64))


@pytest.mark.gpu
def test_attached_writer_streams_u16_output(eng, tmp_path):
    bw, f0, dms, B = np.float32(4e6), np.float32(400e6), [1.0, 2.5], 4
    m = eng.MsosmGpuBatch(bw, dms, f0).initialize(0, B, eng.IN_C64, eng.OUT_U16)
    w = eng.Writer(tmp_path, "obs", dms, B * m.M * 4, slots=3, direct_io=True)
    w.attach_to(m)
    rng = np.random.default_rng(4)
    n = B * m.M
    outs = []
    for _ in range(6):
        x = ((rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 200).astype(np.complex64)
        m.filter_block(x)
        o = np.zeros((len(dms), B * m.M), np.uint32)
        m.get_output(o)
        m.synchronize()
        outs.append(o)
    w.join()
    for d, name in enumerate(w.filenames()):
        np.testing.assert_array_equal(np.fromfile(name, np.uint32), np.concatenate([o[d] for o in outs]))
    w.close()
