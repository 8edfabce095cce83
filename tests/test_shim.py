"""The header-only C++ shim (include/compat) and the psrdada reader, on the CPU.

* A program written against the reference's class interface compiles and links
  against the engine library, and its host-only parts (planning, psrdada
  parsing) run without a GPU.
* Where the reference tree is given (MSOSM_REFERENCE_ROOT), each of the reference's
  five programs (msosm_psrdada.cpp, msosm_save_simulated.cpp and the three benchmark
  mains) compiles and links unchanged against the shim.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import REFERENCE_ROOT, cuda_compile_flags

ROOT = Path(__file__).resolve().parents[1]
COMPAT = ROOT / "include" / "compat"
LIBDIR = ROOT / "acceleratedms-osm_gb300" / "lib"

PROGRAM = r"""
#include "globals.h"
#include "msosm_gpu_batch.h"
#include "osm_gpu_batch.h"
#include "fold_gpu.h"
#include "psrdada.h"
#include <cstdio>

int main(int argc, char **argv)
{
    // Prepare_MSOSM planning through the shim (host only)
    float dms[3] = {1.0f, 2.0f, 3.0f};
    Prepare_MSOSM p(4e6f, dms, 400e6f, 3);
    p.calculate_min_order();
    for (int i = 0; i < 3; i++)
        p.segmentation(i);
    p.generate_dedisp_params(0);
    printf("%d %d %d %d %d %d\n", p.Nd_values[0], p.Nd_values[2], p.M, p.delaycount, p.delay_points[2][0],
           p.delay_points[2][2 * p.M - 1]);
    printf("%.6f %.6f\n", p.dedisp_params[0][0].x, p.dedisp_params[0][0].y);
    Prepare_OSM o(4e6f, 3.0f, 400e6f);
    o.calculate_min_order();
    printf("%lu %lu\n", o.Nd, o.M);
    if (argc > 1)
    {
        PSRDADA f(argv[1]);
        f.initBuffer(4096);
        bool ok = f.readSamples();
        printf("%g %g %d %d %lu %d %u %u\n", f.bw, f.fc, f.nbit, f.npol, f.readCount, (int)ok,
               f.nbit == 16 ? f.pol1_in[0].first : (unsigned)(uint8_t)f.pol1_i8[0],
               f.nbit == 16 ? f.pol2_in[1].second : (unsigned)(uint8_t)f.pol2_i8[3]);
    }
    return 0;
}
"""


def _gxx():
    g = shutil.which("g++")
    if g is None:
        pytest.skip("g++ not available")
    return g


@pytest.fixture(scope="module")
def shim_program(tmp_path_factory, eng):
    d = tmp_path_factory.mktemp("shim")
    src = d / "prog.cpp"
    src.write_text(PROGRAM)
    exe = d / "prog"
    r = subprocess.run([_gxx(), "-std=c++17", "-O1", "-I", str(COMPAT), str(src), "-L", str(LIBDIR), "-lmsosm_gb300",
                        f"-Wl,-rpath,{LIBDIR}", *cuda_compile_flags(), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _dada(path: Path, nbit: int, npol: int, frames: int, rng):
    hdr = f"HDR_VERSION 1.0\nBW 4\nFREQ 402\nNBIT {nbit}\nNCHAN 1\nNDIM 2\nNPOL {npol}\n".encode()
    hdr = hdr + b"\0" * (4096 - len(hdr))
    bytes_per = 4 if nbit == 16 else 2
    body = rng.integers(0, 256, frames * 2048 * bytes_per * npol, dtype=np.uint8).tobytes()
    path.write_bytes(hdr + body)
    return np.frombuffer(body, np.uint8)


def test_shim_planning_matches_oracle(shim_program, orc):
    out = subprocess.run([str(shim_program)], capture_output=True, text=True, check=True).stdout.split("\n")
    nd0, nd2, M, dc, d_first, d_last = map(int, out[0].split())
    plan = orc.Plan(np.float32(4e6), np.float32(400e6), [1.0, 2.0, 3.0], 0, batch=1)
    assert [nd0, nd2] == [plan.nd[0], plan.nd[2]]
    assert (M, dc) == (plan.M, plan.delaycount)
    assert (d_first, d_last) == (plan.delays[2][0], plan.delays[2][-1])
    hx, hy = map(float, out[1].split())
    assert abs(complex(hx, hy) - plan.H[0][0]) < 1e-5
    nd_osm, M_osm = map(int, out[2].split())
    assert nd_osm == orc.osm_nd(np.float32(4e6), np.float32(3.0), np.float32(400e6))
    assert M_osm == orc.osm_min_order(nd_osm)


@pytest.mark.parametrize("nbit,npol", [(16, 1), (16, 2), (8, 2)])
def test_psrdada_reader(shim_program, tmp_path, nbit, npol):
    rng = np.random.default_rng(nbit * 10 + npol)
    f = tmp_path / "obs.dada"
    body = _dada(f, nbit, npol, frames=5, rng=rng)
    out = subprocess.run([str(shim_program), str(f)], capture_output=True, text=True, check=True).stdout
    bw, fc, nb, npl, reads, ok, a, b = out.split("\n")[3].split()
    assert (float(bw), float(fc), int(nb), int(npl)) == (4.0, 402.0, nbit, npol)
    bps = 4 if nbit == 16 else 2
    assert int(reads) == (5 * 2048 * bps * npol) // (npol * 4096 * bps)
    assert int(ok) == 1
    # frame interleaving: pol1 frame 0 starts the body; pol2 frame 0 follows it
    if nbit == 16:
        u = body.view(np.uint16)
        assert int(a) == int(u[0])
        if npol == 2:
            assert int(b) == int(u[2048 * 2 + 3])
    else:
        assert int(a) == int(body[0])
        assert int(b) == int(body[2048 * 2 + 3])


def test_psrdada_rejects_truncated_header(shim_program, tmp_path):
    f = tmp_path / "short.dada"
    f.write_bytes(b"BW 4\n")
    r = subprocess.run([str(shim_program), str(f)], capture_output=True, text=True)
    assert r.returncode != 0 and "header" in r.stderr


REFERENCE_MAINS = ["msosm_psrdada.cpp", "msosm_save_simulated.cpp", "benchmark/check_msosm.cpp",
                   "benchmark/check_osm.cpp", "benchmark/test_msosm_speed.cpp"]


@pytest.mark.skipif(not REFERENCE_ROOT, reason="MSOSM_REFERENCE_ROOT does not name the reference tree")
@pytest.mark.parametrize("main", REFERENCE_MAINS)
def test_reference_main_compiles_against_shim(tmp_path, eng, main):
    src = Path(REFERENCE_ROOT) / main
    assert src.exists(), src
    exe = tmp_path / Path(main).stem
    r = subprocess.run([_gxx(), "-std=c++17", "-O1", "-I", str(COMPAT), str(src), "-L", str(LIBDIR), "-lmsosm_gb300",
                        f"-Wl,-rpath,{LIBDIR}", *cuda_compile_flags(), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
