"""Generate the golden planning fixtures from the reference's own planning code.

Run in a container where the reference tree exists:

    python tests/golden/make_golden.py --ref-root <reference tree> [--segments-only]

It compiles the reference's dedispersion/msosm/msosm_prepare.cpp and
dedispersion/overlap_save/osm_prepare.cpp unmodified (oracle/Makefile target
`ref`, against a project-written FFTW-API shim, since FFTW is not installed),
drives them the way MSOSM_GPU_BATCH::initialize_uint16 and
OSM_GPU_BATCH::initialize_uint16 do (msosm_gpu_batch.cpp:12-93,
osm_gpu_batch.cpp:19-45) and writes what they compute:

  plan_cases.json   Nd per DM, M_min, M, delaycount per DM, the processor-wide
                    delaycount, and every delay map as run-length triples
                    (start, length, delay) -- bit-exact integer pins
  response.npz      the response H (complex64) for the small cases in full and
                    a strided sample + L2 norm for the large ones
  osm_cases.json    Prepare_OSM's Nd / M_min / M for the OSM cases (+ H samples
                    in response.npz)
  segment_cases.json  the reference's own MSOSM_GPU_BATCH::build_segments
                    (msosm_gpu_batch.cpp:262-295, compiled unmodified against stub
                    kernel headers) on every delay map above: segment count and
                    SHA-256 of the int32 (start, len, group) triples per DM, and the
                    full triples of the small cases

The fixtures travel with the repository; the GPU machine never needs the reference.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent

# (name, bandwidth Hz, centre MHz -> f0 = centre - bw/2, DM list, fftpoint, store full H?)
def msosm_cases():
    rng = np.random.default_rng(4)
    c4 = np.sort(np.exp(rng.uniform(np.log(1.0), np.log(1000.0), 1024))).astype(np.float32)
    return [
        # the single-DM workload: 16 MHz at 1400 MHz, DM 50, F = 2^16
        ("c1_dm50_f65536", 16e6, 1400e6, [50.0], 2 ** 16, False),
        # the many-DM workload: 64 MHz at 1400 MHz, 512 DMs linspace(0,200), F = 2^18
        ("c2_512dm_f262144", 64e6, 1400e6, np.linspace(0.0, 200.0, 512).astype(np.float32), 2 ** 18, False),
        ("c2_dm123p4_f262144", 64e6, 1400e6, [123.4], 2 ** 18, False),
        # 2-pol int8 workload: 128 MHz at 820 MHz, 1024 log-uniform DMs (every 16th kept)
        ("c4_64of1024dm_auto", 128e6, 820e6, c4[::16], 0, False),
        # the reference executables' defaults (check_msosm / test_msosm_speed: bw 128 MHz, f0 1 GHz, DM 75)
        ("bench_default_dm75", 128e6, 1e9 + 64e6, [75.0], 0, False),
        # small cases used by the GPU parity tests
        ("small_4mhz_dm1to3", 4e6, 402e6, [1.0, 2.0, 3.0], 0, True),
        ("small_4mhz_dm3_f8192", 4e6, 402e6, [3.0], 8192, True),
        ("small_8mhz_dm0p5to8", 8e6, 604e6, [0.5, 1.0, 2.5, 4.0, 8.0], 0, True),
        ("small_2mhz_tiny", 2e6, 301e6, [0.05, 0.2], 0, True),
        ("psrdada_like_16mhz_dm5_20", 16e6, 1008e6, [5.0, 20.0], 0, False),
    ]


def osm_cases():
    return [
        ("osm_c1_dm50", 16e6, 1400e6, 50.0, 0),
        ("osm_small_dm3", 4e6, 402e6, 3.0, 0),
        ("osm_small_dm1_f8192", 4e6, 402e6, 1.0, 8192),
    ]


def runs(delay: np.ndarray):
    d = np.asarray(delay)
    if d.size == 0:
        return []
    cut = np.flatnonzero(np.diff(d)) + 1
    starts = np.concatenate([[0], cut])
    ends = np.concatenate([cut, [d.size]])
    return [[int(s), int(e - s), int(d[s])] for s, e in zip(starts, ends)]


def segment_fixtures():
    import hashlib

    out = {}
    for name, bw, fc, dms, fftpoint, full_h in msosm_cases():
        bw32 = np.float32(bw)
        f0 = np.float32(np.float32(fc) - np.float32(bw) / np.float32(2))
        r = O.ref_plan(bw32, f0, np.asarray(dms, np.float32), fftpoint, want_delays=True, want_H=False)
        per = []
        for i in range(len(dms)):
            if r["dc"][i] == 0:  # DM 0: the reference leaves the delay map unset
                per.append(None)
                continue
            seg = O.ref_build_segments(r["delays"][i])
            e = dict(count=int(len(seg)), sha256=hashlib.sha256(seg.astype("<i4").tobytes()).hexdigest())
            if full_h:
                e["triples"] = seg.tolist()
            per.append(e)
        out[name] = per
        print(f"{name}: segments per DM {[p['count'] for p in per if p][:4]}...")
    (OUT / "segment_cases.json").write_text(json.dumps(out, separators=(",", ":")))
    print("segment_cases.json", (OUT / "segment_cases.json").stat().st_size, "bytes")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=None, help="the reference tree (default: $MSOSM_REFERENCE_ROOT)")
    ap.add_argument("--segments-only", action="store_true")
    args = ap.parse_args()
    if O.build_ref(args.ref_root) is None:
        raise SystemExit("give the reference tree with --ref-root or MSOSM_REFERENCE_ROOT")
    segment_fixtures()
    if args.segments_only:
        return
    plans = {}
    arrays = {}
    for name, bw, fc, dms, fftpoint, full_h in msosm_cases():
        bw32 = np.float32(bw)
        f0 = np.float32(np.float32(fc) - np.float32(bw) / np.float32(2))
        dms = np.asarray(dms, dtype=np.float32)
        want_h = True
        r = O.ref_plan(bw32, f0, dms, fftpoint, want_delays=True, want_H=want_h)
        F = 2 * r["M"]
        entry = dict(bw=float(bw32), f0=float(f0), dms=[float(x) for x in dms], fftpoint=fftpoint,
                     nd=r["nd"].tolist(), M_min=r["M_min"], M=r["M"], dc=r["dc"].tolist(),
                     delaycount=r["delaycount"],
                     delay_runs=[runs(r["delays"][i]) if r["dc"][i] > 0 else None for i in range(len(dms))])
        plans[name] = entry
        H = r["H"]
        if full_h:
            arrays[f"{name}__H"] = H
        else:
            stride = 257
            idx = np.arange(0, F, stride)
            sel = list(range(min(len(dms), 4)))
            arrays[f"{name}__Hidx"] = idx.astype(np.int32)
            arrays[f"{name}__Hsel"] = np.array(sel, np.int32)
            arrays[f"{name}__Hsample"] = H[sel][:, idx]
            arrays[f"{name}__Hnorm"] = np.linalg.norm(H.astype(np.complex128), axis=1)
        print(f"{name}: M={r['M']} delaycount={r['delaycount']} DMs={len(dms)}")
    osm = {}
    for name, bw, fc, dm, fftpoint in osm_cases():
        bw32 = np.float32(bw)
        f0 = np.float32(np.float32(fc) - np.float32(bw) / np.float32(2))
        r = O.ref_osm_plan(bw32, np.float32(dm), f0, fftpoint, want_H=True)
        M = max(fftpoint // 2, r["M_min"]) if fftpoint else r["M"]
        osm[name] = dict(bw=float(bw32), f0=float(f0), dm=float(np.float32(dm)), fftpoint=fftpoint,
                         nd=r["nd"], M_min=r["M_min"], M=M)
        H = r["H"]
        F = 2 * M
        idx = np.arange(0, F, 131)
        arrays[f"{name}__Hidx"] = idx.astype(np.int32)
        arrays[f"{name}__Hsample"] = H[idx]
        arrays[f"{name}__Hnorm"] = np.array([np.linalg.norm(H.astype(np.complex128))])
        print(f"{name}: Nd={r['nd']} M={M}")
    (OUT / "plan_cases.json").write_text(json.dumps(plans, separators=(",", ":")))
    (OUT / "osm_cases.json").write_text(json.dumps(osm, indent=1))
    np.savez_compressed(OUT / "response.npz", **arrays)
    for p in ("plan_cases.json", "osm_cases.json", "response.npz"):
        print(p, (OUT / p).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
