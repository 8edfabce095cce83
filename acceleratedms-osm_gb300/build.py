"""Build recipe of the MS-OSM engine: nvcc / g++ straight to one shared library.

    python acceleratedms-osm_gb300/build.py        # -> acceleratedms-osm_gb300/lib/libmsosm_gb300.so

Kernels are compiled for sm_103a only (one -gencode), translation units in
parallel; host planning code is compiled with -ffp-contract=off so its float
arithmetic rounds like the reference's.  Objects go to lib/obj (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
OBJ_DIR = LIB_DIR / "obj"
LIB = LIB_DIR / "libmsosm_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["msosm_forward.cu", "msosm_inverse.cu", "msosm_persist.cu", "msosm_fold.cu", "msosm_noalloc.cu", "msosm_tc.cu",
              "msosm_sim.cu"]
CPP_SOURCES = ["msosm_plan.cpp", "msosm_capi.cpp", "msosm_writer.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent / "include"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    jobs = []
    for src in CU_SOURCES:
        s = CSRC / src
        if not s.exists():
            continue
        o = OBJ_DIR / (s.stem + ".o")
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(s), "-o", str(o)])
    cinc = _cuda_include(nvcc)
    for src in CPP_SOURCES:
        s = CSRC / src
        o = OBJ_DIR / (s.stem + ".o")
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                         "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(cinc), "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    objs = [OBJ_DIR / (Path(s).stem + ".o") for s in CU_SOURCES + CPP_SOURCES if (CSRC / s).exists()]
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objs), "-lpthread"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
