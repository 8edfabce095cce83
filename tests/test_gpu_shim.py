"""The C++ drop-in on the GPU: programs written against the reference's classes,
compiled against include/compat and run on the GPU (GPU):

* two fold-mode MSOSM_GPU_BATCH + Fold_GPU's 2-pol intensity and phase fold (the flow
  of msosm_psrdada.cpp:101-146): folded profile against the FP64 oracle's;
* SimulatedComplexSignal's block generator + MSOSM_GPU_BATCH with host output + a fold
  by sample index (the flow of benchmark/check_msosm.cpp:69-190): output and profile
  against the FP64 oracle dedispersing the same generated input;
* SimulatedComplexSignal's impulse generator + MSOSM_DataSave_Uring over three DMs
  (the flow of msosm_save_simulated.cpp:103-150): every per-DM .dat file byte-exact
  against the engine's own uint16 output for the same input.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import cuda_compile_flags, rel_l2

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
                        f"-Wl,-rpath,{LIBDIR}", *cuda_compile_flags(), "-o", str(exe)], capture_output=True, text=True)
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


def _compile(tmp_path, name, text):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / f"{name}.cpp"
    src.write_text(text)
    exe = tmp_path / name
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(COMPAT), str(src), "-L", str(LIBDIR), "-lmsosm_gb300",
                        f"-Wl,-rpath,{LIBDIR}", *cuda_compile_flags(), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


CHECK_PROGRAM = r"""
#include "globals.h"
#include "msosm_gpu_batch.h"
#include "simulated_complex_signal.h"
#include <cstdio>
#include <string>
#include <vector>

// argv: bw f0 dm period fftpoint batch valid_periods outdir
int main(int argc, char **argv)
{
    if (argc != 9)
        return 2;
    const float bw = atof(argv[1]), f0 = atof(argv[2]), period = atof(argv[4]);
    float dm = atof(argv[3]);
    const int fftpoint = atoi(argv[5]), batch = atoi(argv[6]);
    const unsigned long valid = strtoul(argv[7], nullptr, 10);
    const std::string dir = argv[8];

    MSOSM_GPU_BATCH proc(bw, &dm, f0, 1);
    proc.initialize_uint16(fftpoint, batch);
    const unsigned long M = proc.M, step = (unsigned long)batch * M;
    const unsigned long block = (unsigned long)(period * bw);
    // skip the windows whose overlap history is the zero start, then whole periods
    const unsigned long fold_start = ((M + block - 1) / block) * block;
    const unsigned long steps = (fold_start + valid * block + step - 1) / step;
    const unsigned long periods = (steps * step + block - 1) / block;

    SimulatedComplexSignal sig(bw, dm, f0, period, "uint16");
    sig.generate_pulsar_signal_block(periods - valid, valid);
    CUDA_CHECK(cudaHostRegister(sig.signal_u16, sig.signal_size * sizeof(uint16_pair), cudaHostRegisterDefault));
    std::vector<uint16_pair> out(steps * step);
    for (unsigned long k = 0; k < steps; k++)
    {
        proc.filter_block_uint16(sig.signal_u16 + k * step);
        proc.get_output(out.data() + k * step);
    }
    proc.synchronize();

    std::vector<double> prof(block, 0.0);
    for (unsigned long p = 0; p < valid; p++)
        for (unsigned long i = 0; i < block; i++)
        {
            const uint16_pair &v = out[fold_start + p * block + i];
            const double re = (double)v.first - 32768.0 * (v.first != 0);
            const double im = (double)v.second - 32768.0 * (v.second != 0);
            prof[i] += std::sqrt(re * re + im * im) / (double)valid;
        }
    FILE *f = fopen((dir + "/in.u16").c_str(), "wb");
    fwrite(sig.signal_u16, sizeof(uint16_pair), steps * step, f);
    fclose(f);
    f = fopen((dir + "/out.u16").c_str(), "wb");
    fwrite(out.data(), sizeof(uint16_pair), steps * step, f);
    fclose(f);
    f = fopen((dir + "/prof.f64").c_str(), "wb");
    fwrite(prof.data(), sizeof(double), block, f);
    fclose(f);
    CUDA_CHECK(cudaHostUnregister(sig.signal_u16));
    printf("dims %lu %lu %lu %lu %lu\n", M, step, steps, block, fold_start);
    return 0;
}
"""


def test_check_msosm_shaped_program_on_the_gpu(eng, orc, tmp_path):
    exe = _compile(tmp_path, "check_prog", CHECK_PROGRAM)
    bw, f0, dm, period, B, valid = np.float32(8e6), np.float32(1000e6), np.float32(20.0), np.float32(0.004), 32, 8
    run = subprocess.run([str(exe), str(float(bw)), str(float(f0)), str(float(dm)), str(float(period)), "0", str(B),
                          str(valid), str(tmp_path)], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    dims = [l for l in run.stdout.splitlines() if l.startswith("dims")][0].split()[1:]
    M, step, steps, block, fold_start = map(int, dims)
    x = np.fromfile(tmp_path / "in.u16", np.uint32)
    out = np.fromfile(tmp_path / "out.u16", np.uint32)
    prof = np.fromfile(tmp_path / "prof.f64", np.float64)
    assert x.size == out.size == steps * step and prof.size == block

    plan = orc.Plan(bw, f0, [float(dm)], 0, batch=B)
    assert plan.M == M
    om = orc.Msosm(plan, B, fp64=True)
    ref = np.concatenate([om.process(orc.decode_u16(x[k * step:(k + 1) * step]))[0].reshape(-1) for k in range(steps)])
    # uint16 output: the oracle's series encoded the same way, within one code
    enc = orc.encode_u16(ref.astype(np.complex64))
    d_re = np.abs((out & 0xFFFF).astype(np.int64) - (enc & 0xFFFF).astype(np.int64))
    d_im = np.abs((out >> 16).astype(np.int64) - (enc >> 16).astype(np.int64))
    assert max(d_re.max(), d_im.max()) <= 1
    assert np.mean((d_re == 0) & (d_im == 0)) > 0.999
    # the folded |x| profile against the oracle's float series folded the same way
    seg = ref[fold_start:fold_start + valid * block].reshape(valid, block)
    ref_prof = np.abs(seg).mean(axis=0)
    assert rel_l2(prof, ref_prof) < 2e-3
    # the test pulse's main component comes back at phase 0.5
    smooth = np.convolve(prof, np.ones(64) / 64, mode="same")
    assert abs(np.argmax(smooth) / block - 0.5) < 0.03


SAVE_PROGRAM = r"""
#include "globals.h"
#include "simulated_complex_signal.h"
#include "msosm_data_save_uring.h"
#include <cstdio>
#include <string>

// argv: bw f0 period batch outdir dm0 dm1 dm2
int main(int argc, char **argv)
{
    if (argc != 9)
        return 2;
    const float bw = atof(argv[1]), f0 = atof(argv[2]), period = atof(argv[3]);
    const int batch = atoi(argv[4]);
    const std::string dir = argv[5];
    float dms[3] = {(float)atof(argv[6]), (float)atof(argv[7]), (float)atof(argv[8])};

    MSOSM_DataSave_Uring proc(bw, dms, f0, 3);
    proc.initialize_uint16(0, batch);
    const unsigned long step = (unsigned long)batch * proc.M;
    const unsigned long block = (unsigned long)(period * bw);
    const unsigned long repeat = (3 * step + block - 1) / block;
    SimulatedComplexSignal sig(bw, dms[0], f0, period, "uint16");
    sig.generate_pulsar_signal(repeat, false, 0, false);
    const unsigned long count = sig.signal_size / step;

    proc.config_save(dir, "simulated");
    proc.initialize_uring(4, count);
    proc.start_saving();
    for (unsigned long k = 0; k < count; k++)
    {
        proc.filter_block_uint16(sig.signal_u16 + k * step);
        proc.copy_to_slot();
    }
    proc.join_saving();
    FILE *f = fopen((dir + "/in.u16").c_str(), "wb");
    fwrite(sig.signal_u16, sizeof(uint16_pair), count * step, f);
    fclose(f);
    printf("dims %lu %lu\n", step, count);
    return 0;
}
"""


def test_save_simulated_shaped_program_on_the_gpu(eng, tmp_path):
    exe = _compile(tmp_path, "save_prog", SAVE_PROGRAM)
    bw, f0, period, B = np.float32(8e6), np.float32(1000e6), np.float32(0.004), 16
    dms = [10.0, 20.0, 30.0]
    out_dir = tmp_path / "dat"
    out_dir.mkdir()
    run = subprocess.run([str(exe), str(float(bw)), str(float(f0)), str(float(period)), str(B), str(out_dir),
                          *map(str, dms)], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    step, count = map(int, [l for l in run.stdout.splitlines() if l.startswith("dims")][0].split()[1:])
    assert count >= 3
    x = np.fromfile(out_dir / "in.u16", np.uint32)
    m = eng.MsosmGpuBatch(bw, dms, f0).initialize(0, B, eng.IN_U16, eng.OUT_U16)
    want = np.zeros((count, len(dms), step), np.uint32)
    buf = np.zeros((len(dms), step), np.uint32)
    for k in range(count):
        m.filter_block(np.ascontiguousarray(x[k * step:(k + 1) * step]))
        m.get_output(buf)
        m.synchronize()
        want[k] = buf
    files = sorted(out_dir.glob("simulated_DM*.dat"), key=lambda p: float(p.stem.split("DM")[1]))
    assert [p.name for p in files] == ["simulated_DM10.00.dat", "simulated_DM20.00.dat", "simulated_DM30.00.dat"]
    for d, p in enumerate(files):
        got = np.fromfile(p, np.uint32)
        assert got.size == count * step
        assert np.array_equal(got, want[:, d, :].reshape(-1)), p.name


DADA_PROGRAM = r"""
#include "globals.h"
#include "msosm_gpu_batch.h"
#include "fold_gpu.h"
#include "psrdada.h"
#include <cstdio>
#include <vector>

// argv: dada file, dm, batch, period, bins.  The msosm_psrdada.cpp flow: the reader's
// header gives the band; two polarisations dedispersed, 2-pol intensity folded.  NBIT 16
// runs the reference's classes; NBIT 8 the C ABI's int8 input on the same engine.
int main(int argc, char **argv)
{
    if (argc != 6)
        return 2;
    float dm = atof(argv[2]);
    const int batch = atoi(argv[3]);
    const float period = atof(argv[4]);
    const unsigned long bins = strtoul(argv[5], nullptr, 10);
    PSRDADA f(argv[1]);
    const float bw = f.bw * 1e6f, f0 = (f.fc - f.bw / 2) * 1e6f;
    msosm_t *h[2];
    for (int p = 0; p < 2; p++)
    {
        msosm_compat::check(msosm_create(bw, f0, &dm, 1, &h[p]), nullptr, "create");
        msosm_compat::check(msosm_init(h[p], 0, batch, f.nbit == 8 ? MSOSM_IN_I8 : MSOSM_IN_U16, MSOSM_OUT_C64), h[p],
                            "init");
    }
    int M = 0;
    msosm_get_dims(h[0], &M, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    const unsigned long n = (unsigned long)batch * M;
    Fold_GPU fold(period, bw, n, "fold_dada.txt", bins);
    f.initBuffer(n);
    printf("M %d reads %lu\n", M, f.readCount);
    for (unsigned long r = 0; r < f.readCount; r++)
    {
        if (!f.readSamples())
            return 3;
        const void *p1 = f.nbit == 8 ? (const void *)f.pol1_i8 : (const void *)f.pol1_in;
        const void *p2 = f.nbit == 8 ? (const void *)f.pol2_i8 : (const void *)f.pol2_in;
        msosm_compat::check(msosm_process(h[0], p1, nullptr), h[0], "process");
        msosm_compat::check(msosm_process(h[1], p2, nullptr), h[1], "process");
        msosm_compat::check(msosm_fold_accumulate(fold.handle(), msosm_device_output(h[0]), msosm_device_output(h[1]),
                                                  nullptr), nullptr, "fold");
    }
    msosm_sync(h[0], nullptr);
    fold.get_folded_data();
    for (unsigned long k = 0; k < fold.time_bin; k++)
        printf("%.9g\n", fold.folded_data[k]);
    msosm_destroy(h[0]);
    msosm_destroy(h[1]);
    return 0;
}
"""


@pytest.mark.parametrize("nbit", [16, 8])
def test_psrdada_file_through_the_engine(eng, orc, tmp_path, nbit):
    exe = _compile(tmp_path, "dada_prog", DADA_PROGRAM)
    bw_mhz, fc_mhz, dm, B, period, K = 16.0, 1008.0, 5.0, 8, 0.0041, 64
    bw, f0 = np.float32(bw_mhz * 1e6), np.float32((fc_mhz - bw_mhz / 2) * 1e6)
    m = eng.MsosmGpuBatch(bw, [dm], f0).initialize(0, B, eng.IN_C64, eng.OUT_C64)
    n = B * m.M
    reads = 3
    rng = np.random.default_rng(nbit)
    pols = []
    for _ in range(2):
        iq = np.clip(np.round(rng.normal(0, 20, (reads * n, 2))), -127, 127).astype(np.int64)
        pols.append(iq)
    # body: frames of 2048 samples, pol 1 frame k then pol 2 frame k
    frames = reads * n // 2048
    if nbit == 16:
        words = [((p[:, 0] + 32768) | ((p[:, 1] + 32768) << 16)).astype(np.uint32) for p in pols]
        body = np.stack([w.reshape(frames, 2048) for w in words], axis=1).reshape(-1).tobytes()
    else:
        b8 = [p.astype(np.int8).reshape(frames, 2048 * 2) for p in pols]
        body = np.stack(b8, axis=1).reshape(-1).tobytes()
    hdr = (f"HDR_VERSION 1.0\nBW {bw_mhz}\nFREQ {fc_mhz}\nNBIT {nbit}\nNCHAN 1\nNDIM 2\nNPOL 2\n").encode()
    f = tmp_path / f"obs{nbit}.dada"
    f.write_bytes(hdr + b"\0" * (4096 - len(hdr)) + body)
    run = subprocess.run([str(exe), str(f), str(dm), str(B), str(period), str(K)], capture_output=True, text=True,
                         cwd=tmp_path, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    lines = run.stdout.splitlines()
    assert lines[0] == f"M {m.M} reads {reads}"
    got = np.array([float(v) for v in lines[1:]])

    plan = orc.Plan(bw, f0, [dm], 0, batch=B)
    oms = [orc.Msosm(plan, B, fp64=True) for _ in range(2)]
    s_ = np.zeros(K)
    c_ = np.zeros(K, np.uint64)
    dt = 1.0 / float(bw)
    for r in range(reads):
        xs = [(p[r * n:(r + 1) * n, 0] + 1j * p[r * n:(r + 1) * n, 1]).astype(np.complex64) for p in pols]
        ya = oms[0].process(xs[0])[0].reshape(-1)
        yb = oms[1].process(xs[1])[0].reshape(-1)
        orc.fold(orc.intensity2(ya, yb), K, r * n * dt, dt, float(np.float32(period)), s_, c_)
    ref = orc.fold_finalize(s_, c_)
    assert rel_l2(got, ref) < 1e-4
