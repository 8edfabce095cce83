#!/usr/bin/env python
"""Throughput benchmark of the MS-OSM hot path on GB300.

Workload (the many-DM configuration): complex64 single-pol baseband, 64 MHz
bandwidth at 1400 MHz centre (f0 = 1368 MHz), 2^26 samples with a pulsar
(period 33 ms, 5 % duty, -10 dB per-sample SNR) injected at DM 123.4; 512 DM
trials uniformly spaced in 0..200 pc/cm^3; FFT size 2^18 (M = 2^17), batch 32
windows per call; every trial folded into 512 phase bins (no series output).

One "step" = one pass of the engine over the whole 2^26-sample baseband
(16 calls of 2^22 samples), all 512 trials dedispersed and folded.

  value   samples x DM trials per second with the input resident in HBM
          (CUDA events on the launch stream, max over ranks).
  e2e     the same through the C ABI with the input in pinned HOST memory:
          every step copies its 512 MB in and reads the folded profiles back.
  roofline  the dominant kernel's achieved bandwidth under the algorithmic
          byte model of 16 B per sample x DM, from per-launch CUDA events taken
          inside the timed region, against the measured HBM copy bandwidth.
  cpu_baseline  the FP32 CPU port of the same algorithm (oracle/) on a bounded
          sample, all host threads.
  reference_gpu_design  the reference's GPU design (cuFFT forward, gather x
          response, batched cuFFT inverse, discard + fold) restated in
          baseline/cufft_pipeline and timed on the same workload (off with
          --no-cufft-baseline).

Other workloads: --workload single_dm_50 (1 DM at 16 MHz, F = 2^16) and
--workload two_pol_1024 (2-pol int8, 1024 log-uniform DMs, F = 2^20, fused 2-pol
fold); --samples / --dm-trials / --batch shrink or reshape a workload for captures.

`--impl reference` times that CPU implementation alone (the reference has no
CPU MS-OSM path of its own; its planning code is x86-build-only here).
Multi-GPU (torchrun): each rank dedisperses its own interleaved share of a
512*N-trial grid (weak scaling, no data-path collective); the host-side barrier
and the max-over-ranks reduction use gloo.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "acceleratedms-osm_gb300"))

METRIC = "baseband samples/s x DM trials"
UNIT = "sample*DM/s"
BYTES_PER_UNIT = 16  # algorithmic bytes per sample x DM, fold-only: the spectra read once per trial

WORKLOADS = {
    "many_dm_512": dict(bw=64e6, centre=1400e6, n_dms=512, dm_lo=0.0, dm_hi=200.0, fftpoint=1 << 18, batch=32,
                        nbins=512, samples=1 << 26, period=0.033, inject_dm=123.4, snr_db=-10.0, duty=0.05),
    "single_dm_50": dict(bw=16e6, centre=1400e6, n_dms=1, dm_lo=50.0, dm_hi=50.0, fftpoint=1 << 16, batch=32,
                         nbins=256, samples=1 << 22, period=0.033, inject_dm=50.0, snr_db=-10.0, duty=0.05),
    # 2-pol int8 I/Q (Gaussian, sigma 20, clipped), 1024 DMs log-uniform in 1..1000 (seed 4,
    # sorted), which forces F = 2^20; the fused 2-pol fold (msosm_attach_fold_pol2); 8 windows
    # per call (2 / 4 / 8 / 16 measured 6.13 / 6.19 / 6.29 / 6.36e10 on 256 DMs, fewer response
    # re-reads; at full size 8 gave 6.39e10 and 16 6.31e10)
    "two_pol_1024": dict(bw=128e6, centre=820e6, n_dms=1024, dm_lo=1.0, dm_hi=1000.0, dm_dist="loguniform",
                         fftpoint=1 << 20, batch=8, nbins=256, samples=1 << 28, period=0.0071, pols=2, sigma=20.0),
    # DM refinement: 64 simulated sources of 2^20..2^24 samples (log-uniform, seed 5), true
    # DMs uniform in 10..300, guesses 0.5 DM off, 20 steps each on the smoothed sharpness
    # (pymsosm.refine); 16 MHz at 1400 MHz, 2 ms period, 2 % Gaussian pulse, -10 dB
    "refine_64": dict(bw=16e6, centre=1400e6, n_sources=64, len_lo=20, len_hi=24, dm_lo=10.0, dm_hi=300.0,
                      offset=0.5, period=0.002, duty=0.02, snr_db=-10.0, nbins=256),
}


def dm_grid(w, rank=0, world=1):
    if w["n_dms"] == 1:
        return np.array([w["dm_lo"]], np.float32)
    if w.get("dm_dist") == "loguniform":
        rng = np.random.default_rng(4)
        g = np.sort(np.exp(rng.uniform(np.log(w["dm_lo"]), np.log(w["dm_hi"]), w["n_dms"] * world)))
        g = g.astype(np.float32)
    else:
        g = np.linspace(w["dm_lo"], w["dm_hi"], w["n_dms"] * world).astype(np.float32)
    return np.ascontiguousarray(g[rank::world])


def f0_of(w):
    return np.float32(np.float32(w["centre"]) - np.float32(w["bw"]) / np.float32(2))


# ----------------------------------------------------------------------------
def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profile_traffic(kernel: str):
    """DRAM bytes per F-point transform of `kernel` from the committed ncu summary."""
    p = ROOT / "profiles" / "traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.f = None

    def _gpu_id(self):
        try:
            import torch

            p = torch.cuda.get_device_properties(self.dev)
            return f"{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0"
        except Exception:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
            return vis.split(",")[self.dev] if vis else str(self.dev)

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self._gpu_id()], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.f is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def reduce_max(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_profiles(folded: np.ndarray, world: int) -> np.ndarray:
    """The per-rank [D][K] folded profiles of an interleaved DM share (dm_grid), gathered
    on the host into the whole grid's [D * world][K] in grid order (row i from rank
    i % world).  Every rank gets the result; this is the only exchange of the sharded
    path, after the timed region."""
    if world <= 1:
        return folded
    import torch.distributed as dist

    parts = [None] * world
    dist.all_gather_object(parts, np.ascontiguousarray(folded))
    full = np.empty((sum(p.shape[0] for p in parts), folded.shape[1]), folded.dtype)
    for r, p in enumerate(parts):
        full[r::world] = p
    return full


# ----------------------------------------------------------------------------
def cpu_port_rate(w, n_dms_sample: int, substeps: int, seed: int = 3, steps: int = 1, warmup: int = 0):
    """FP32 CPU port (oracle/) on a bounded sample: returns (rate, seconds, description)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    oracle.build()
    bw, f0 = np.float32(w["bw"]), f0_of(w)
    grid = dm_grid(w)
    pick = np.linspace(0, len(grid) - 1, min(n_dms_sample, len(grid))).round().astype(int)
    dms = grid[np.unique(pick)]
    plan = oracle.Plan(bw, f0, dms, w["fftpoint"], batch=w["batch"])
    m = oracle.Msosm(plan, w["batch"], fp64=False, H=plan.H.astype(np.complex64))
    m.set_fold(w["nbins"], np.float32(w["period"]), bw)
    n = w["batch"] * plan.M
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    for _ in range(warmup):
        m.process(x, want_output=False)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        for _ in range(substeps):
            m.process(x, want_output=False)
        times.append(time.perf_counter() - t0)
    units = substeps * n * len(dms)
    sec = float(np.mean(times))
    desc = (f"{len(dms)} of the {len(grid)} DM trials x {substeps} calls of {n} samples "
            f"({units:.3g} sample*DM), FP32, fold-only, {m.nthreads} threads")
    return units / sec, sec, desc, m.nthreads, times


L2_FLUSH_BYTES = 256 << 20  # twice the GB300's L2


def fits_in_l2(w) -> bool:
    """Baseband + responses of one step small enough to stay in L2 between steps."""
    pols = w.get("pols", 1)
    in_bytes = 2 * pols * w["samples"] if pols == 2 else 8 * w["samples"]
    return in_bytes + w["n_dms"] * w["fftpoint"] * 8 <= 129e6


def workload_config(args, w, world):
    """The "config" object of a workload, printed identically by both arms (the engine's
    launch geometry goes to a separate "launch" key)."""
    bw, f0 = np.float32(w["bw"]), f0_of(w)
    F = w["fftpoint"]
    pols = w.get("pols", 1)
    in_bytes = 2 * pols * w["samples"] if pols == 2 else 8 * w["samples"]
    resp_bytes = w["n_dms"] * F * 8
    cfg = {"workload": args.workload, "dm_trials_per_gpu": w["n_dms"], "fft_size": F, "M": F // 2,
           "batch": w["batch"], "phase_bins": w["nbins"], "bandwidth_hz": float(bw), "f0_hz": float(f0)}
    if pols == 2:
        cfg.update({"pols": 2, "samples_per_pol": w["samples"], "input": "int8 I/Q, 2 pols"})
    else:
        cfg.update({"precision": args.precision, "samples": w["samples"], "input": "complex64, 1 pol"})
    cfg["l2"] = (f"inputs larger than L2 ({in_bytes / 2**20:.0f} MB baseband, "
                 f"{pols} x {resp_bytes / 2**20:.0f} MB responses)" if not fits_in_l2(w) else
                 f"inputs of {(in_bytes + resp_bytes) / 2**20:.0f} MB: L2 flushed between timed steps "
                 f"({L2_FLUSH_BYTES >> 20} MB written, outside the timed spans)")
    cfg["parallelism"] = f"dm-shard x{world}"
    return cfg


def run_reference(args, w, rank, world):
    if rank != 0:
        return
    if "n_sources" in w:
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no DM refinement"}))
        return
    n_dms_sample = 32
    substeps = 2
    rate, sec, desc, cores, times = cpu_port_rate(w, n_dms_sample, substeps, steps=args.steps, warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, w, world),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference implements MS-OSM only on the GPU (cuFFT); its CPU implementation of the path "
                 "is the project's FP32 restatement of the same algorithm (oracle/), timed here"),
    }
    print(json.dumps(line))


# ----------------------------------------------------------------------------
CUFFT_LIB = ROOT / "baseline" / "cufft_pipeline" / "lib" / "libmsosm_cufft_pipeline.so"


def cufft_design_rate(proc, dms, dinp, w, calls, steps, stream):
    """The reference's GPU design (cuFFT forward, delayed-bin gather x response, batched
    cuFFT inverse, discard + fold) restated in baseline/cufft_pipeline and timed on the same
    workload, device-resident input, CUDA events; the engine's plan tables are reused."""
    import ctypes as C

    import torch

    if not CUFFT_LIB.exists():
        return {"unavailable": f"{CUFFT_LIB.relative_to(ROOT)} not built"}
    L = C.CDLL(str(CUFFT_LIB))
    L.mcp_create.argtypes = [C.c_int] * 6 + [C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]
    L.mcp_process.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcp_read.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.mcp_reset_fold.argtypes = [C.c_void_p, C.c_void_p]
    L.mcp_destroy.argtypes = [C.c_void_p]
    dev = dinp.device
    D, F, M, B = len(dms), proc.fftpoint, proc.M, proc.batch
    H = torch.empty((D, F), dtype=torch.complex64, device=dev)
    dl = torch.empty((D, F), dtype=torch.int16, device=dev)
    for i in range(D):
        H[i] = torch.from_numpy(proc.response(i))
        dl[i] = torch.from_numpy(proc.delay_points(i).astype(np.uint16).view(np.int16))
    chunk = 64
    h = C.c_void_p()
    rc = L.mcp_create(int(np.log2(F)), B, D, proc.ring_blocks, chunk, w["nbins"], np.float32(w["period"]),
                      np.float32(w["bw"]), H.data_ptr(), dl.data_ptr(), C.byref(h))
    if rc != 0:
        return {"unavailable": f"mcp_create failed ({rc})"}
    sp = C.c_void_p(stream.cuda_stream)
    try:
        def step():
            L.mcp_reset_fold(h, sp)
            for c in range(calls):
                rc = L.mcp_process(h, C.c_void_p(dinp.data_ptr() + c * B * M * 8), sp)
                if rc != 0:
                    raise RuntimeError(f"mcp_process failed ({rc})")

        step()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        t_ms = ev0.elapsed_time(ev1)
        sums = np.zeros((D, w["nbins"]))
        cnts = np.zeros((D, w["nbins"]), np.uint64)
        L.mcp_read(h, sums.ctypes.data, cnts.ctypes.data)
    finally:
        L.mcp_destroy(h)
    folded = sums / np.maximum(cnts, 1)
    return {"value": calls * B * M * D * steps / (t_ms * 1e-3), "unit": UNIT, "ms_per_step": t_ms / steps,
            "kind": "the reference's cuFFT pipeline restated (baseline/cufft_pipeline): cuFFT forward, "
                    "gather x response, batched cuFFT inverse in DM chunks of %d, fused discard + fold" % chunk,
            "timed": "before the engine's launches, with no L2 set aside for persisting lines", "_folded": folded}


def reference_shaped_rate(eng, bw, f0, dms, w, dinp, calls, steps, stream):
    """The engine used the way the reference's programs use their processor: the series of
    every DM written (complex64, fold mode), then a separate fold pass over it (Fold_GPU's
    calculate_intensity + fold_data_phase), instead of the fused fold-only transform.  Same
    workload, device-resident input, CUDA events."""
    import torch

    p = eng.MsosmGpuBatch(bw, dms, f0).initialize(w["fftpoint"], w["batch"], eng.IN_C64, eng.OUT_C64)
    n = p.batch * p.M
    fold = eng.FoldGpu(np.float32(w["period"]), bw, n, w["nbins"], len(dms))

    def step():
        fold.reset(stream)
        for c in range(calls):
            p.filter_block(dinp[2 * c * n:2 * (c + 1) * n], stream)
            fold.accumulate(p.get_output_pointer(), None, stream)

    step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    t_ms = e0.elapsed_time(e1)
    del p, fold
    return {"value": calls * n * len(dms) * steps / (t_ms * 1e-3), "unit": UNIT, "ms_per_step": t_ms / steps,
            "kind": "series of every DM to HBM (complex64), then the stand-alone fold over it"}


def int8_baseband(n, sigma, seed):
    """n complex samples of int8 interleaved I/Q: N(0, sigma^2) rounded, clipped to +-127."""
    rng = np.random.default_rng(seed)
    out = np.empty(2 * n, np.int8)
    step = 1 << 24
    for i in range(0, 2 * n, step):
        v = rng.standard_normal(min(step, 2 * n - i), dtype=np.float32) * np.float32(sigma)
        out[i:i + len(v)] = np.clip(np.rint(v), -127, 127).astype(np.int8)
    return out


def run_two_pol(args, w, rank, world, local):
    """Two polarisations of int8 baseband, every DM trial, fused 2-pol fold: per call the
    first polarisation's transform writes |a|^2 and the second's folds sqrt(|a|^2+|b|^2)."""
    import torch

    import pymsosm as eng

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    bw, f0 = np.float32(w["bw"]), f0_of(w)
    dms = dm_grid(w, rank, world)
    N = w["samples"]
    hosts = [torch.from_numpy(int8_baseband(N, w["sigma"], 40 + 2 * rank + p)).pin_memory() for p in range(2)]
    devs = [h.to(dev) for h in hosts]
    procs = [eng.MsosmGpuBatch(bw, dms, f0).initialize(w["fftpoint"], w["batch"], eng.IN_I8, eng.OUT_NONE)
             .set_launch_shape(args.ctas_per_sm, args.dm_group) for _ in range(2)]
    step_n = procs[0].batch * procs[0].M
    calls = N // step_n
    fold = eng.FoldGpu(np.float32(w["period"]), bw, step_n, w["nbins"], len(dms))
    procs[0].attach_fold_pol2(procs[1], fold)
    stream = torch.cuda.current_stream(dev)
    bpc = 2 * step_n  # int8 bytes per call and pol

    def step(src):
        for c in range(calls):
            procs[0].filter_block(src[0][c * bpc:(c + 1) * bpc], stream)
            procs[1].filter_block(src[1][c * bpc:(c + 1) * bpc], stream)

    for _ in range(args.warmup):
        step(devs)
    torch.cuda.synchronize()
    for p in procs:
        p.profile_reset()
        p.profile(True)
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step(devs)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    for p in procs:
        p.profile(False)
    t_ms = reduce_max(ev0.elapsed_time(ev1), world)
    units_rank = 2 * N * len(dms)  # samples per pol x pols x DM trials
    total_units = reduce_sum(units_rank * args.steps, world)
    value = total_units / (t_ms * 1e-3)
    profs = [p.profile_read() for p in procs]
    launches = sum(v["launches"] for pr in profs for v in pr.values())
    dom = "inv_persistent"
    ms = sum(pr[dom]["ms"] for pr in profs)
    timed = sum(pr[dom]["timed"] for pr in profs)
    trans = sum(pr[dom]["transforms"] for pr in profs) / max(sum(pr[dom]["launches"] for pr in profs), 1)
    per_launch_ms = ms / max(timed, 1)
    bytes_per_launch = BYTES_PER_UNIT * procs[0].M * trans
    peak, peak_src = measured_peak()
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": bytes_per_launch / (per_launch_ms * 1e-3) / 1e9, "peak": peak,
        "unit": "GB/s", "frac": bytes_per_launch / (per_launch_ms * 1e-3) / 1e9 / peak, "peak_source": f"of {peak_src}",
        "traffic": (tr * trans) if (tr := profile_traffic("inv_persistent_two_pol")) is not None else None,
        "traffic_note": "ncu DRAM bytes of the second polarisation's (fused-fold) launch per transform, "
                        "scaled to this launch's transforms",
        "bytes_per_launch": bytes_per_launch, "ms_per_launch": per_launch_ms,
        "pipeline_achieved": BYTES_PER_UNIT * units_rank * args.steps / (t_ms * 1e-3) / 1e9,
    }
    # end to end from pinned host memory, one pass over both polarisations per step
    folded = np.zeros((len(dms), w["nbins"]), np.float32)
    step(hosts)
    fold.read_folded(folded, stream)
    barrier(world)
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        fold.reset(stream)
        step(hosts)
        fold.read_folded(folded, stream)
    torch.cuda.synchronize()
    e_ms = reduce_max((time.perf_counter() - e0) * 1e3, world)
    e2e = {"value": total_units / (e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(2 * hosts[0].numel()),
           "d2h_bytes_per_step": int(folded.nbytes)}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, w, world), "launch": procs[1].launch_info(),
        "clocks": clk.summary(), "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
        "check": {"folded_finite": bool(np.isfinite(folded).all()), "dm_range": [float(dms[0]), float(dms[-1])]},
    }
    if world == 1 and not args.no_cpu_baseline:
        rate, sec, desc, cores, _ = cpu_port_rate(w, 16, 2)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": desc + ", one polarisation (the per-pol cost of the 2-pol path)"}
    print(json.dumps(line))


def run_engine(args, w, rank, world, local):
    import torch

    import pymsosm as eng
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    bw, f0 = np.float32(w["bw"]), f0_of(w)
    dms = dm_grid(w, rank, world)
    N = w["samples"]

    # the baseband comes from the engine's GPU pulsar simulator (msosm_sim_*)
    sim = eng.Simulator(bw, f0, np.float32(w["inject_dm"]), np.float32(w["period"]), kind=eng.SIM_GAUSSIAN,
                        duty=w["duty"], snr_db=w["snr_db"], seed=2 + rank)
    dc = torch.empty(N, dtype=torch.complex64, device=dev)
    sim.generate(N, out=dc)
    torch.cuda.synchronize()
    del sim
    dinp = dc.view(torch.float32)
    host = dinp.cpu().pin_memory()

    proc = eng.MsosmGpuBatch(bw, dms, f0).initialize(w["fftpoint"], w["batch"], eng.IN_C64, eng.OUT_NONE)
    proc.set_launch_shape(args.ctas_per_sm, args.dm_group)
    proc.set_precision(PRECISIONS[args.precision])
    step_n = proc.batch * proc.M
    calls = N // step_n
    fold = eng.FoldGpu(np.float32(w["period"]), bw, step_n, w["nbins"], len(dms))
    proc.attach_fold(fold)
    stream = torch.cuda.current_stream(dev)

    def step(src):
        proc.filter_blocks(src, calls, stream)

    # the cuFFT restatement of the reference's GPU design, timed before the engine's
    # launches with the L2 persisting set-aside back at zero
    base = None
    if world == 1 and not args.no_cufft_baseline:
        eng.reset_l2_persisting()  # the simulator's filter launches set L2 aside for their own ring
        base = cufft_design_rate(proc, dms, dinp, w, calls, args.steps, stream)
        torch.cuda.synchronize()

    # warm-up (also compiles nothing: kernels are prebuilt)
    for _ in range(args.warmup):
        step(dinp)
    torch.cuda.synchronize()

    # ---- timed region: device-resident input ------------------------------
    proc.profile_reset()
    proc.profile(True)
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if fits_in_l2(w):
        # a step's inputs would stay in L2: time each step alone and overwrite L2
        # between steps, outside the timed spans
        scrub = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clk:
            for a0, a1 in evs:
                scrub.zero_()
                a0.record(stream)
                step(dinp)
                a1.record(stream)
            torch.cuda.synchronize()
        t_ms = sum(a0.elapsed_time(a1) for a0, a1 in evs)
        del scrub
    else:
        with ClockSampler(local) as clk:
            ev0.record(stream)
            for _ in range(args.steps):
                step(dinp)
            ev1.record(stream)
            torch.cuda.synchronize()
        t_ms = ev0.elapsed_time(ev1)
    barrier(world)
    proc.profile(False)
    t_ms = reduce_max(t_ms, world)
    units_per_step_rank = N * len(dms)
    total_units = reduce_sum(units_per_step_rank * args.steps, world)
    value = total_units / (t_ms * 1e-3)
    prof = proc.profile_read()
    launches = sum(v["launches"] for v in prof.values())

    # roofline of the dominant kernel (largest summed device time)
    dom = max(prof, key=lambda k: prof[k]["ms"])
    pk = prof[dom]
    per_launch_ms = pk["ms"] / max(pk["timed"], 1)
    trans_per_launch = pk["transforms"] / max(pk["launches"], 1)
    bytes_per_launch = BYTES_PER_UNIT * proc.M * trans_per_launch
    achieved = bytes_per_launch / (per_launch_ms * 1e-3) / 1e9
    peak, peak_src = measured_peak()
    tr = profile_traffic(dom)
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": f"of {peak_src}",
        "traffic": (tr * trans_per_launch) if tr is not None else None,
        "bytes_per_launch": bytes_per_launch, "ms_per_launch": per_launch_ms,
        "pipeline_achieved": BYTES_PER_UNIT * units_per_step_rank * args.steps / (t_ms * 1e-3) / 1e9,
        "kernel_share": {k: v["ms"] / max(sum(p["ms"] for p in prof.values()), 1e-9) for k, v in prof.items()},
    }

    # ---- the same steps replayed from a captured CUDA graph (msosm_graph_*) --
    # (needs the ring's period in steps to divide the calls of a step: 2 here)
    try:
        graph = proc.capture(dinp, calls)
    except eng.MsosmError as err:  # the ring's period does not divide this step's calls
        graph, graph_line = None, {"unavailable": str(err)}
    if graph is not None:
        graph.launch(stream)
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(args.steps):
            graph.launch(stream)
        g1.record(stream)
        torch.cuda.synchronize()
        g_ms = reduce_max(g0.elapsed_time(g1), world)
        graph_line = {"value": total_units / (g_ms * 1e-3), "unit": UNIT, "ms_per_step": g_ms / args.steps,
                      "calls_per_graph": calls,
                      "note": "each step's forward passes and persistent inverse launches replayed from one graph"}
        del graph

    # ---- end-to-end through the C ABI from pinned host memory -------------
    folded_host = np.zeros((len(dms), w["nbins"]), np.float32)
    proc.filter_blocks(host, calls, stream)  # one untimed e2e warm-up step
    fold.read_folded(folded_host, stream)
    barrier(world)
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        fold.reset(stream)  # each step folds exactly one pass over the baseband
        proc.filter_blocks(host, calls, stream)
        fold.read_folded(folded_host, stream)  # D2H of the step's result (synchronises)
    torch.cuda.synchronize()
    e_ms = (time.perf_counter() - e0) * 1e3
    barrier(world)
    e_ms = reduce_max(e_ms, world)
    e2e = {"value": total_units / (e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(host.numel() * 4),
           "d2h_bytes_per_step": int(folded_host.nbytes)}

    # ---- sanity: the injected DM is recovered ------------------------------
    def snr(p):
        base = np.median(p)
        mad = np.median(np.abs(p - base)) * 1.4826
        return float((p.max() - base) / mad) if mad > 0 else 0.0

    # the whole grid's profiles on every rank (host gather of the DM shards)
    all_folded = gather_profiles(folded_host, world)
    all_dms = dm_grid(w, 0, 1) if world == 1 else np.sort(np.concatenate(
        [dm_grid(w, r, world) for r in range(world)]))
    s = np.array([snr(p) for p in all_folded])
    best = int(np.argmax(s))
    check = {"best_dm": float(all_dms[best]), "snr_best": float(s[best]), "snr_dm_lowest": float(s[0]),
             "injected_dm": w["inject_dm"], "dm_trials_gathered": int(len(all_folded))}

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[args.precision], "data": "synthetic",
        "config": workload_config(args, w, world), "launch": proc.launch_info(),
        "clocks": clk.summary(), "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "check": check,
        "graph": graph_line,
    }
    if world == 1 and not args.no_cufft_baseline:
        line["reference_shaped_form"] = reference_shaped_rate(eng, bw, f0, dms, w, dinp, calls, args.steps, stream)
    if base is not None:
        if "_folded" in base:
            f = base.pop("_folded")
            base["folded_rel_l2_vs_engine"] = float(np.linalg.norm(f - folded_host) / np.linalg.norm(folded_host))
        line["reference_gpu_design"] = base
    if world == 1 and not args.no_cpu_baseline:
        rate, sec, desc, cores, _ = cpu_port_rate(w, 64, 4)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    print(json.dumps(line))


def run_refine(args, w, rank, world, local):
    """The differentiation workload: every source refined from its guess (20 steps on the
    smoothed sharpness, two many-DM comb passes per source).  A step of the bench is the
    refinement of all sources; the metric counts the samples x DM trials the comb passes
    dedisperse."""
    import torch

    import pymsosm as eng
    from pymsosm import refine as R

    torch.cuda.set_device(local)
    bw, f0 = np.float32(w["bw"]), f0_of(w)
    rng = np.random.default_rng(5)
    ns = w["n_sources"]
    lengths = np.exp2(rng.uniform(w["len_lo"], w["len_hi"], ns)).astype(np.int64)
    true = rng.uniform(w["dm_lo"], w["dm_hi"], ns)
    guess = true + np.where(rng.random(ns) < 0.5, -w["offset"], w["offset"])
    mine = list(range(rank, ns, world))
    srcs = {}
    for i in mine:
        sim = eng.Simulator(bw, f0, np.float32(true[i]), np.float32(w["period"]), kind=eng.SIM_GAUSSIAN,
                            duty=w["duty"], snr_db=w["snr_db"], seed=1000 + i)
        srcs[i] = sim.generate(int(lengths[i]))
    trials = [2 * int(round(st.half_width / st.spacing)) + 1 for st in R.DEFAULT_STAGES]

    def one_pass():
        return {i: R.refine_dm(srcs[i], bw, f0, guess[i], np.float32(w["period"]), w["nbins"])[0] for i in mine}

    for _ in range(args.warmup):
        one_pass()
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            est = one_pass()
        torch.cuda.synchronize()
        t_s = time.perf_counter() - t0
    barrier(world)
    t_s = reduce_max(t_s, world)
    units = reduce_sum(float(sum(int(lengths[i]) for i in mine) * sum(trials) * args.steps), world)
    err = np.array([est[i] - true[i] for i in mine])
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": units / t_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_s * 1e3 / args.steps, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (GPU pulsar simulator)",
        "config": {"workload": args.workload, "sources": ns, "samples_per_source": [int(v) for v in lengths],
                   "comb_trials_per_stage": trials, "gradient_steps": sum(st.steps for st in R.DEFAULT_STAGES),
                   "bandwidth_hz": float(bw), "f0_hz": float(f0), "period_s": w["period"],
                   "timing": "host wall clock around whole refinements (planning, simulation excluded)",
                   "parallelism": f"source-shard x{world}"},
        "clocks": clk.summary(),
        "refinement": {"initial_offset_dm": w["offset"], "rms_error_dm": float(np.sqrt(np.mean(err ** 2))),
                       "max_abs_error_dm": float(np.abs(err).max()),
                       "within_0p1_dm": int((np.abs(err) < 0.1).sum()), "sources_on_rank0": len(mine)},
    }
    print(json.dumps(line))


# inverse-transform arithmetic (msosm_set_precision) and the JSON dtype label of each
PRECISIONS = {"fp32": 0, "bf16x3": 1, "fp16x3": 2}
DTYPES = {"fp32": "f32", "bf16x3": "bf16x3 (hi/lo operands, f32 accumulate)",
          "fp16x3": "f16x3 (hi/lo operands, f32 accumulate)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="many_dm_512", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cufft-baseline", action="store_true",
                    help="skip timing the cuFFT restatement of the reference's GPU design")
    ap.add_argument("--samples", type=int, default=0, help="override the baseband length (profiling captures)")
    ap.add_argument("--dm-trials", type=int, default=0, help="override the DM-trial count (profiling captures)")
    ap.add_argument("--batch", type=int, default=0, help="override the windows per call")
    ap.add_argument("--ctas-per-sm", type=int, default=0,
                    help="cap on resident CTAs per SM of the persistent transform (0 = as many as fit)")
    ap.add_argument("--dm-group", type=int, default=0,
                    help="DM trials per window-major group of the persistent transform's order (0 = default)")
    ap.add_argument("--precision", default="fp32", choices=sorted(PRECISIONS),
                    help="inverse-transform arithmetic: fp32 register DFTs, or tensor-core DFT stages on "
                         "split bf16/fp16 operands (bf16x3 / fp16x3)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    w = dict(WORKLOADS[args.workload])
    if args.samples and "samples" in w:
        w["samples"] = args.samples
    if args.dm_trials:
        w["n_dms"] = args.dm_trials
    if args.batch:
        w["batch"] = args.batch
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, w, rank, world)
    elif "n_sources" in w:
        run_refine(args, w, rank, world, local)
    elif w.get("pols", 1) == 2:
        run_two_pol(args, w, rank, world, local)
    else:
        run_engine(args, w, rank, world, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
