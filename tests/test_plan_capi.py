"""Product host logic and the C-ABI library, without a GPU.

The engine's own planning code (acceleratedms-osm_gb300/csrc/msosm_plan.cpp),
reached through the host-only C-ABI entry points, must reproduce the reference's
integer planning bit-for-bit (golden fixtures from the reference build) and its
response to FP32 rounding.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import expand_runs, rel_l2


def test_library_exports_every_declared_symbol(eng):
    L = eng.lib()
    declared = eng.declared_functions()
    assert len(declared) >= 30
    missing = [f for f in declared if not hasattr(L, f)]
    assert not missing, missing
    assert b"sm_103a" in L.msosm_version()


def test_planning_matches_reference(eng, golden_plans):
    for name, c in golden_plans.items():
        nd = eng.plan_nd(c["bw"], c["f0"], c["dms"])
        assert nd.tolist() == c["nd"], name
        mmin = eng.plan_min_order(nd)
        assert mmin == c["M_min"], name
        M = c["M"]
        F = 2 * M
        dcs = []
        for i, dm in enumerate(c["dms"]):
            d, dc = eng.plan_segmentation(c["bw"], c["f0"], dm, int(nd[i]), M)
            dcs.append(dc)
            runs = c["delay_runs"][i]
            if runs is None:
                assert dc == 0 and not d.any()
            else:
                np.testing.assert_array_equal(d, expand_runs(runs, F), err_msg=f"{name} DM#{i}")
        assert dcs == c["dc"], name


def test_osm_planning_matches_reference(eng, golden_osm):
    for name, c in golden_osm.items():
        nd, mmin = eng.osm_plan(c["bw"], c["dm"], c["f0"])
        assert nd == c["nd"] and mmin == c["M_min"], name


def test_response_matches_reference_and_oracle(eng, orc, golden_plans, golden_arrays):
    for name, c in golden_plans.items():
        M = c["M"]
        if f"{name}__H" in golden_arrays:
            for i, dm in enumerate(c["dms"]):
                H = eng.plan_response(c["bw"], c["f0"], dm, M)
                assert rel_l2(H, golden_arrays[f"{name}__H"][i]) < 2e-6, (name, i)
                assert rel_l2(H, orc.response(c["bw"], c["f0"], dm, M)) < 2e-7, (name, i)
        elif M <= (1 << 19):
            idx = golden_arrays[f"{name}__Hidx"]
            for k, i in enumerate(golden_arrays[f"{name}__Hsel"][:2]):
                H = eng.plan_response(c["bw"], c["f0"], c["dms"][i], M)
                assert rel_l2(H[idx], golden_arrays[f"{name}__Hsample"][k]) < 5e-6, (name, i)


def test_create_rejects_bad_arguments(eng):
    L = eng.lib()
    h = C.c_void_p()
    dms = np.array([5.0, 1.0], np.float32)  # descending: the reference reads out of bounds
    assert L.msosm_create(16e6, 1e9, dms.ctypes.data, 2, C.byref(h)) == 1
    dms = np.array([-1.0], np.float32)
    assert L.msosm_create(16e6, 1e9, dms.ctypes.data, 1, C.byref(h)) == 1
    assert L.msosm_create(16e6, 1e9, dms.ctypes.data, 0, C.byref(h)) == 1
    assert L.msosm_status_string(5) == b"unsupported configuration"


def test_create_computes_nd_on_host(eng, golden_plans):
    c = golden_plans["c2_512dm_f262144"]
    m = eng.MsosmGpuBatch(c["bw"], c["dms"], c["f0"])
    assert m.nd.tolist() == c["nd"]
    # process before init is a state error, not a crash
    with pytest.raises(eng.MsosmError):
        m.filter_block(np.zeros(4, np.uint32))


def test_header_is_plain_c_and_links(tmp_path, eng):
    """include/msosm_gb300.h is the C boundary: strict C99 compiles against it and a C
    program links the library and runs the host-only planning entry points."""
    import shutil
    import subprocess
    from pathlib import Path

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    root = Path(__file__).resolve().parents[1]
    lib = root / "acceleratedms-osm_gb300" / "lib"
    src = tmp_path / "probe.c"
    src.write_text(r"""
#include <stdio.h>
#include "msosm_gb300.h"
int main(void)
{
    float dms[2] = {1.0f, 2.0f};
    int nd[2] = {0, 0};
    if (msosm_plan_nd(4e6f, 400e6f, dms, 2, nd) != MSOSM_OK)
        return 1;
    printf("%s %d %d\n", msosm_status_string(MSOSM_ERR_ARG), nd[0], nd[1]);
    return 0;
}
""")
    exe = tmp_path / "probe"
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", str(root / "include"),
                        str(src), "-L", str(lib), "-lmsosm_gb300", f"-Wl,-rpath,{lib}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    words = run.stdout.split()
    assert int(words[-2]) > 0 and int(words[-1]) > int(words[-2])
