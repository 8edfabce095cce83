"""The C++ drop-in on the GPU: a program written against the reference's classes
(MSOSM_GPU_BATCH in fold mode for two polarisations, Fold_GPU's 2-pol intensity and
phase fold -- the flow of msosm_psrdada.cpp:101-146) compiled against include/compat and
run on the GPU; its folded profile must match the FP64 oracle's (GPU)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
COMPAT = ROOT / "include" / "compat"
LIBDIR = ROOT / "acceleratedms-osm_gb300" / "lib"

PROGRAM = r"""
#include "globals.h"
#include "msosm_gpu_batch.h"
#include "fold_gpu.h"
#include <cstdio>
#include <cstdlib>
#include <vector>

// argv: data file (pol1 blocks then pol2 blocks, uint16 pairs), bw, f0, dm, fftpoint,
// batch, steps, period, bins
int main(int argc, char **argv)
{
    if (argc != 10)
        return 2;
    const float bw = atof(argv[2]), f0 = atof(argv[3]);
    float dm = atof(argv[4]);
    const int fftpoint = atoi(argv[5]), batch = atoi(argv[6]), steps = atoi(argv[7]);
    const float period = atof(argv[8]);
    const unsigned long bins = strtoul(argv[9], nullptr, 10);
    MSOSM_GPU_BATCH p1(bw, &dm, f0, 1), p2(bw, &dm, f0, 1);
    p1.initialize_uint16(fftpoint, batch, true);
    p2.initialize_uint16(fftpoint, batch, true);
    const unsigned long n = (unsigned long)batch * p1.M;
    Fold_GPU fold(period, bw, n, "fold_shim.txt", bins);
    std::vector<uint16_pair> a(n), b(n);
    FILE *f = fopen(argv[1], "rb");
    if (!f)
        return 3;
    for (int s = 0; s < steps; s++)
    {
        fseek(f, (long)(s * n * sizeof(uint16_pair)), SEEK_SET);
        if (fread(a.data(), sizeof(uint16_pair), n, f) != n)
            return 4;
        fseek(f, (long)((steps + s) * n * sizeof(uint16_pair)), SEEK_SET);
        if (fread(b.data(), sizeof(uint16_pair), n, f) != n)
            return 4;
        p1.filter_block_uint16(a.data());
        p2.filter_block_uint16(b.data());
        fold.calculate_intensity(&p1, &p2); // pulls get_output_pointer(), as the reference's does
        fold.fold_data_phase();
    }
    fclose(f);
    fold.get_folded_data();
    printf("M %lu\n", (unsigned long)p1.M);
    for (unsigned long i = 0; i < bins; i++)
        printf("%.9g\n", fold.folded_data[i]);
    return 0;
}
"""


def test_reference_shaped_2pol_program_on_the_gpu(eng, orc, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "prog.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "prog"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(COMPAT), str(src), "-L", str(LIBDIR), "-lmsosm_gb300",
                        f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    bw, f0, dm, F, B, steps, period, K = np.float32(16e6), np.float32(1000e6), 20.0, 1 << 16, 4, 3, 0.0052, 128
    M = F // 2
    n = B * M
    rng = np.random.default_rng(31)
    pols = []
    for _ in range(2):
        iq = np.clip(np.round(rng.normal(0, 20, (steps * n, 2))), -127, 127).astype(np.int32) + 32768
        pols.append((iq[:, 0] | (iq[:, 1] << 16)).astype(np.uint32))
    data = tmp_path / "pols.u16"
    np.concatenate(pols).tofile(data)
    run = subprocess.run([str(exe), str(data), str(float(bw)), str(float(f0)), str(dm), str(F), str(B), str(steps),
                          str(period), str(K)], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    lines = [l for l in run.stdout.splitlines() if l and not l.startswith("FFT point")]
    assert lines[0] == f"M {M}"
    got = np.array([float(x) for x in lines[1:]])

    plan = orc.Plan(bw, f0, [dm], F, batch=B)
    oms = [orc.Msosm(plan, B, fp64=True) for _ in range(2)]
    s_ = np.zeros(K)
    c_ = np.zeros(K, np.uint64)
    dt = 1.0 / float(bw)
    for s in range(steps):
        xa = oms[0].process(orc.decode_u16(pols[0][s * n:(s + 1) * n]))[0].reshape(-1)
        xb = oms[1].process(orc.decode_u16(pols[1][s * n:(s + 1) * n]))[0].reshape(-1)
        orc.fold(orc.intensity2(xa, xb), K, s * n * dt, dt, float(np.float32(period)), s_, c_)
    ref = orc.fold_finalize(s_, c_)
    assert rel_l2(got, ref) < 1e-4
