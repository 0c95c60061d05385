#!/usr/bin/env python
"""Benchmark of the GB300 photon-transport engine.

Headline workload (one "step"): the two-phase fluorescence simulation of the
voxelized heterogeneous medium — 200 x 200 x 100 voxels of 0.02 cm, 8 labels,
seeded spheres and cylinders with a fp32 fluorophore map — 1e8 excitation
photons from a Gaussian beam with the 3D photon hitting density, then the
emission phase with PHOTONS_PER_VOXEL photons from every emitting voxel, R/T
images at both wavelengths.  The metric is photons per second (excitation +
emission photons).

  value       batched engine, medium and tallies resident in HBM, CUDA-event
              timed per step on the engine's stream, L2 flushed between steps
  e2e         the same through the C ABI with host buffers: medium upload,
              run, every image and the fluence copied back, each step
  plain       the same simulation with the emission phase as one launch per
              emitting voxel (the reference's schedule), timed on a sample
  exact_stepping  voxel-boundary stepping against the reference's stepping on
              the same medium at a tenth of the budgets
  batching   256 Gaussian beams on a 16 x 16 raster over the 4 x 4 x 2 cm
              sphere medium, log-uniform budgets 1e6..5e7 (3.1e9 photons;
              --batching-scale scales them), one persistent launch vs one
              launch per beam
  serving     Poisson stream of requests with their own media (64^3 ..
              256 x 256 x 128) and 1e5..1e8 photons at ~80 % load through the
              continuous-batching server: p50/p99 latency, photons/s
  precision   the config-5 medium (512 x 512 x 256 voxels, 268 MB map), the
              FP32 builds against the FP64 build of the same kernel on the
              same seeds: integrated R/T/absorbed error and z, R image
  cpu_baseline  the reference's transport algorithm (the oracle restatement in
              reference-stream mode, bit-identical to the reference's code) on
              the host cores, on a bounded sample of the same workload

--impl reference times that CPU implementation alone.  The reference's own
CUDA program is not run: this repository holds none of the reference's
sources, so there is nothing of it to build where the benchmark runs.
"""
from __future__ import annotations

import argparse
import csv
import hashlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "photons/s, two-phase fluorescence MC (excitation + emission), voxelized heterogeneous medium"
UNIT = "photons/s"
EXC_PHOTONS = 100_000_000
PHOTONS_PER_VOXEL = 1000
WORKLOAD = ("voxelized heterogeneous bulk descriptor 200x200x100 @0.02cm, 8 labels, seeded spheres+cylinders "
            "with fp32 fluorophore map; 1e8 excitation photons (Gaussian beam) with 3D photon hitting density, "
            "emission phase 1000 photons per emitting voxel; R/T images 100x100 @0.04cm at both wavelengths")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ traffic

TRAFFIC_FILE = os.path.join(ROOT, "profiles", "transport_fast_traffic.json")
KERNEL_SOURCES = ("transport.cuh", "transport_fast.cu", "engine_types.h", "portable_math.h")


def kernel_source_sha() -> str:
    """SHA-256 over the fast-math transport kernel's sources and nvcc flags
    (include paths left out): the identity of the build a DRAM-traffic
    capture belongs to."""
    from cudamcfl_gb300 import build as b
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(b.CSRC, f), "rb") as fh:
            h.update(fh.read())
    flags = b.ARCH + [f for f in b.NVCC_COMMON if not f.startswith("-I")] + b.CUDA_UNITS["transport_fast.cu"]
    h.update(" ".join(flags).encode())
    return h.hexdigest()


_UNITS = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "Tbyte": 1e12,
          "nsecond": 1e-9, "usecond": 1e-6, "msecond": 1e-3, "second": 1.0,
          "ns": 1e-9, "us": 1e-6, "ms": 1e-3, "s": 1.0}


def traffic_from_csv(path: str, command: str) -> dict:
    """Per transport launch of an ncu CSV capture (--csv with the metrics
    dram__bytes_read.sum, dram__bytes_write.sum, gpu__time_duration.sum):
    DRAM bytes and duration; written to TRAFFIC_FILE with the build's source
    hash."""
    launches = {}
    with open(path, newline="") as f:
        rows = [r for r in csv.reader(f) if r]
    head = next(i for i, r in enumerate(rows) if "Metric Name" in r)
    cols = rows[head]
    ci = {k: cols.index(k) for k in ("ID", "Kernel Name", "Metric Name", "Metric Unit", "Metric Value")}
    for r in rows[head + 1:]:
        if len(r) < len(cols) or "mcfl_transport_fast" not in r[ci["Kernel Name"]]:
            continue
        v = float(r[ci["Metric Value"]].replace(",", "")) * _UNITS.get(r[ci["Metric Unit"]], 1.0)
        d = launches.setdefault(int(r[ci["ID"]]), {"kernel": r[ci["Kernel Name"]]})
        d[r[ci["Metric Name"]]] = v
    out = []
    for i in sorted(launches):
        d = launches[i]
        out.append({"launch": len(out), "kernel": d["kernel"][:80],
                    "dram_bytes": d.get("dram__bytes_read.sum", 0.0) + d.get("dram__bytes_write.sum", 0.0),
                    "duration_s": d.get("gpu__time_duration.sum")})
    rec = {"source_sha256": kernel_source_sha(), "command": command, "launches": out,
           "dram_bytes_per_launch": sum(x["dram_bytes"] for x in out) / max(1, len(out))}
    with open(TRAFFIC_FILE, "w") as f:
        json.dump(rec, f, indent=1)
        f.write("\n")
    return rec


def traffic_of_this_build():
    """(DRAM bytes per transport launch, note) from TRAFFIC_FILE when it was
    captured on this build's kernel sources, else (None, why)."""
    try:
        with open(TRAFFIC_FILE) as f:
            rec = json.load(f)
    except (OSError, ValueError):
        return None, "no ncu capture of the DRAM traffic on record"
    if rec.get("source_sha256") != kernel_source_sha():
        return None, "the DRAM-traffic capture on record belongs to another build of the kernel"
    return rec["dram_bytes_per_launch"], f"ncu capture of this build: {rec['command']}"


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clock and throttle-reason samples while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int = 0):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        busy = [s for s in sm if s > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


# ------------------------------------------------------------------ CPU arm

def cpu_reference_sample(nthreads: int, exc_photons: int = 4_000_000, fl_voxels: int = 16, per_voxel: int = 40_000):
    """The reference's transport algorithm on host threads over the benchmark
    medium (reference RNG streams and relaunch schedule, C-library math).
    Returns (photons/s, photons, seconds, description, excitation passes per
    photon, per-phase rates: excitation-only and emission-only photons/s and
    passes/s)."""
    from cudamcfl_gb300 import media
    from oracle import pyoracle
    pyoracle.build()
    o = pyoracle.Oracle()
    m = media.config2(seed=2)
    nz, ny, nx = m.labels.shape
    vc = m.voxel_cm
    sim = pyoracle.sim_from_arrays(
        m.labels, m.bulks, half_x=float(np.float32(nx * vc[0] / 2)), half_y=float(np.float32(ny * vc[1] / 2)),
        thickness=float(np.float32(nz * vc[2])), vox_per_cm=[float(np.float32(1 / v)) for v in vc],
        photons=exc_photons, per_voxel=per_voxel, det=(0.04, 0.04, 100, 100, 0.0, 0.0), fluor_map=m.fluor_map,
        do_fl=1 if fl_voxels > 0 else 0)
    sim.max_fl_voxels = fl_voxels
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        sp = os.path.join(d, "safeprimes_base32.txt")
        o.write_safeprimes(sp, 32769)
        t0 = time.perf_counter()
        r = o.run_refstream(sim, sp, 12345, 777, libm=True, nthreads=nthreads)
        dt = time.perf_counter() - t0
    photons = r.photons_exc + r.photons_fl
    desc = (f"config-2 medium, {r.photons_exc} excitation photons + {r.fl_voxels} emitting voxels x {per_voxel} "
            f"emission photons; reference RNG streams (32768 MWC) and relaunch schedule, libm math")
    phases = {"excitation_photons_per_s": r.photons_exc / r.seconds_exc if r.seconds_exc > 0 else None,
              "excitation_passes_per_s": r.steps_exc / r.seconds_exc if r.seconds_exc > 0 else None,
              "emission_photons_per_s": r.photons_fl / r.seconds_fl if r.seconds_fl > 0 and r.photons_fl else None,
              "emission_passes_per_s": r.steps_fl / r.seconds_fl if r.seconds_fl > 0 and r.photons_fl else None,
              "excitation_seconds": r.seconds_exc, "emission_seconds": r.seconds_fl,
              "passes_per_photon_fl": r.steps_fl / max(1, r.photons_fl)}
    return photons / dt, photons, dt, desc, r.steps_exc / max(1, r.photons_exc), phases


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference_sample(nthreads, exc_photons=100_000, fl_voxels=1)
    vals, tot_p, tot_t = [], 0, 0.0
    desc, ppp, phases = "", 0.0, {}
    for _ in range(args.steps):
        v, p, t, desc, ppp, phases = cpu_reference_sample(nthreads, exc_photons=600_000, fl_voxels=4)
        vals.append(v)
        tot_p += p
        tot_t += t
    value = tot_p / tot_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": desc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": desc,
                         "passes_per_photon_exc": ppp, "phases_last_step": phases},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--math", default="fast", choices=["fast", "exact"])
    ap.add_argument("--batching-scale", type=float, default=1.0,
                    help="batching section: scale of config3's per-beam budgets (1e6..5e7 at 1.0)")
    ap.add_argument("--skip", default="",
                    help="comma list of sections to skip: plain,exact_stepping,batching,serving,precision,cpu,e2e")
    ap.add_argument("--precision-photons", type=float, default=1e8,
                    help="precision section: photons per build (config5, FP32 builds vs FP64)")
    ap.add_argument("--profile", action="store_true",
                    help="small case for ncu: the benchmark medium, --photons excitation photons and --per-voxel "
                         "emission photons per voxel, --warmup runs then one run (2 transport launches per run)")
    ap.add_argument("--photons", type=int, default=2_000_000)
    ap.add_argument("--variant", type=int, default=0, help="--profile: kernel variant (0..2)")
    ap.add_argument("--per-voxel", type=int, default=20, help="--profile: emission photons per emitting voxel")
    ap.add_argument("--exact-stepping", action="store_true", help="--profile: voxel-boundary stepping")
    ap.add_argument("--traffic-from", default="",
                    help="write the DRAM traffic per transport launch of an ncu CSV capture (with this build's "
                         "source hash) to profiles/transport_fast_traffic.json and exit; --traffic-command names "
                         "the captured command")
    ap.add_argument("--traffic-command", default="")
    ap.add_argument("--express-period", type=int, default=0,
                    help="serving: one warp in this many draws the express queue first (0: the server's default)")
    ap.add_argument("--express-ratio", type=int, default=0,
                    help="serving: express requests are at most 1/ratio of the head's remaining (0: default)")
    ap.add_argument("--pass-form", type=int, default=0,
                    help="--profile: 0 the pass arranged for the SIMT warp, 1 every test as its own branch")
    ap.add_argument("--relaunch", type=int, default=0,
                    help="--profile: free lanes of a warp that start new photons together (0: the context's)")
    ap.add_argument("--phd-agg", type=int, default=0,
                    help="--profile: hitting-density tally, 0 one add per pass, 1 register sums, 2 warp sums")
    args = ap.parse_args()
    if args.traffic_from:
        print(json.dumps(traffic_from_csv(args.traffic_from, args.traffic_command)))
        return 0
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.profile:
        return profile_case(args)

    import torch
    import cudamcfl_gb300 as mc
    from cudamcfl_gb300 import build, media

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    skip = set(s for s in args.skip.split(",") if s)
    build.build()
    math_mode = mc.MATH_FAST if args.math == "fast" else mc.MATH_EXACT
    stream = torch.cuda.Stream()
    ctx = mc.Context(device=local, math=math_mode)
    ctx.set_stream(stream.cuda_stream)
    lib = mc.load()

    m = media.config2(seed=2)
    med = ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
    # replicas only: every rank simulates its own photon streams (seeded by rank)
    rd = mc.run_desc(EXC_PHOTONS, det=m.det, photons_per_voxel=PHOTONS_PER_VOXEL, fluence=1,
                     seed_exc=1 + 1000 * rank, seed_fl=2 + 1000 * rank)
    stats_out = mc.RunOut()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def one_step():
        return lib.mcfl_run(ctx.handle, med.handle, mc.ctypes.byref(rd), mc.ctypes.byref(stats_out))

    # launch shape: time every kernel variant on a 1.6e7-photon sample, keep
    # the fastest (on 4e6-photon samples the excitation launch's choice did
    # not carry over to the full budget: more of a small sample is launch
    # tail)
    variant, tune_rate = ctx.autotune(med, rd, sample_photons=16_000_000)

    for _ in range(args.warmup):
        mc.check(one_step())
    torch.cuda.synchronize()
    launches0 = ctx.launches
    clocks = ClockSampler(local).start()
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms, photons_step, exc_ms, fl_ms = [], [], [], []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)  # L2 flush (512 MB > 129 MB L2) outside the timed events
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        mc.check(one_step())
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        photons_step.append(EXC_PHOTONS + stats_out.photons_fl)
        exc_ms.append(stats_out.ms_exc)
        fl_ms.append(stats_out.ms_fl)
    torch.cuda.synchronize()
    if dist:
        torch.distributed.barrier()
    clk = clocks.stop()
    launches = ctx.launches - launches0
    total_ms = sum(step_ms)
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * sum(photons_step) / (total_ms / 1e3)
    se, sf = dict(zip(mc.STAT_NAMES, stats_out.stats_exc)), dict(zip(mc.STAT_NAMES, stats_out.stats_fl))
    exc_steps_per_photon = se["steps"] / EXC_PHOTONS
    fl_steps_per_photon = sf["steps"] / max(1, stats_out.photons_fl)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "photons_per_step": photons_step[0], "excitation_photons": EXC_PHOTONS,
                   "emitting_voxels": stats_out.fl_voxels, "emission_photons": stats_out.photons_fl,
                   "math": args.math, "l2": "flushed between steps (512 MB write)", "parallelism": "replicas only",
                   "schedule": "batched: one persistent launch per phase, CUDA-graph replay",
                   "variant": variant, "variant_emission": ctx.get_option("variant_fl"),
                   "pass_form": ctx.get_option("pass_form"),
                   "block": ctx.get_option("launch_block"), "grid": ctx.get_option("grid"),
                   "regs": ctx.get_option("regs"), "l2_window": ctx.get_option("l2_window"),
                   "phd_agg": ctx.get_option("phd_agg"), "relaunch": ctx.get_option("relaunch"),
                   "autotune_sample_photons_per_s": tune_rate},
        "phases": {"excitation_ms": statistics.mean(exc_ms), "emission_ms": statistics.mean(fl_ms),
                   "excitation_photons_per_s": EXC_PHOTONS / (statistics.mean(exc_ms) / 1e3),
                   "emission_photons_per_s": stats_out.photons_fl / (statistics.mean(fl_ms) / 1e3),
                   "steps_per_photon": {"excitation": exc_steps_per_photon, "emission": fl_steps_per_photon},
                   "transport_steps_per_s": (se["steps"] + sf["steps"]) / (statistics.mean(step_ms) / 1e3),
                   "energy_residual": stats_out.energy_exc[3]},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank != 0:
        if dist:
            torch.distributed.destroy_process_group()
        return 0

    # --- roofline of the dominant kernel (the transport kernel) ---
    # Algorithmic work per transport pass, counted from the reference's
    # source (CUDAMCFLtransport.cu:286-447,585-625): 10 MUFU (log, sin, cos,
    # 2 sqrt, rsqrt, 4 reciprocals) + 8 conversions on the XU pipe (16 lanes
    # per SM per clock), ~60 FP32 operations on the FMA pipes (128 lanes).
    # achieved = ops per launch / mean launch time (CUDA events around each
    # transport launch inside the replayed graph); the larger fraction is the
    # bound.
    xu_ops, fp32_ops = 18, 60
    passes = se["steps"] + sf["steps"]
    launch_s = (statistics.mean(exc_ms) + statistics.mean(fl_ms)) / 1e3
    pass_rate = passes / launch_s
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    sm_mhz = peaks.get("sm_max_mhz", 2070.0)
    n_sm = ctx.get_option("sm_count")
    xu_peak = n_sm * 16 * sm_mhz * 1e6
    fp32_peak = n_sm * 128 * sm_mhz * 1e6
    # DRAM bytes per transport launch of this workload, from an ncu capture
    # of this build's kernel (keyed by its source hash), else null
    traffic, traffic_note = traffic_of_this_build()
    result["roofline"] = {
        "bound": "xu", "achieved": xu_ops * pass_rate / 1e12, "peak": xu_peak / 1e12, "unit": "Top/s",
        "frac": xu_ops * pass_rate / xu_peak, "traffic": traffic,
        "fp32": {"achieved": fp32_ops * pass_rate / 1e12, "peak": fp32_peak / 1e12,
                 "frac": fp32_ops * pass_rate / fp32_peak},
        "passes_per_s": pass_rate,
        "note": (f"neither HBM nor tensor cores bound this kernel (no contraction; medium and tallies L2-resident): "
                 f"algorithmic XU ops ({xu_ops}: 10 MUFU + 8 conversions) per transport pass x passes/s over "
                 f"{n_sm} SMs x 16 XU lanes x {sm_mhz:.0f} MHz (sm_max_mhz of MEASURED_PEAKS.json); FP32 analogue "
                 f"({fp32_ops} ops/pass over 128 lanes) beside it; traffic = mean DRAM bytes per transport launch "
                 f"({traffic_note})"),
    }

    # --- e2e through the C ABI with host buffers ---
    if "e2e" not in skip:
        nv = m.labels.size
        xy = 100 + 100 * 100
        bufs = {k: np.zeros(n, dtype=dt) for k, n, dt in (
            ("Rd", xy, np.uint64), ("Tt", xy, np.uint64), ("R", xy, np.float64), ("T", xy, np.float64),
            ("phd", nv, np.float64), ("flR", xy, np.float64), ("flT", xy, np.float64))}
        out = mc.RunOut()
        out.Rd, out.Tt = mc.u64ptr(bufs["Rd"]), mc.u64ptr(bufs["Tt"])
        out.R, out.T, out.phd = mc.f64ptr(bufs["R"]), mc.f64ptr(bufs["T"]), mc.f64ptr(bufs["phd"])
        out.flR, out.flT = mc.f64ptr(bufs["flR"]), mc.f64ptr(bufs["flT"])
        d, keep = mc._medium_desc(m.labels, m.bulks, m.voxel_cm, m.fluor_map)
        h2d = m.labels.nbytes + m.fluor_map.nbytes + 3 * 16 * len(m.bulks) + 2 * 256
        d2h = sum(b.nbytes for b in bufs.values()) + 8 * (2 * mc.NSTATS + 4)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ph = 0
        for _ in range(args.steps):
            h = mc.ctypes.c_void_p()
            mc.check(lib.mcfl_medium_create(ctx.handle, mc.ctypes.byref(d), mc.ctypes.byref(h)))
            mc.check(lib.mcfl_run(ctx.handle, h, mc.ctypes.byref(rd), mc.ctypes.byref(out)))
            lib.mcfl_medium_free(h)
            ph += EXC_PHOTONS + out.photons_fl
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        result["e2e"] = {"value": ph / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                         "d2h_bytes_per_step": int(d2h)}

    # --- plain schedule of the same simulation (emission: one launch per voxel) ---
    if "plain" not in skip:
        sample = 400
        r = mc.run_plain(ctx, med, rd, max_voxels=sample)
        per_voxel_ms = r["ms_fl"] / max(1, r["fl_voxels"])
        plain_ms = r["ms_exc"] + per_voxel_ms * stats_out.fl_voxels
        plain_value = (EXC_PHOTONS + stats_out.photons_fl) / (plain_ms / 1e3)
        result["plain"] = {"value": plain_value, "unit": UNIT, "ms_per_step": plain_ms,
                           "sample": f"excitation + first {r['fl_voxels']} of {stats_out.fl_voxels} emitting voxels, "
                                     f"one launch + host wait per voxel; {per_voxel_ms:.3f} ms per voxel",
                           "batched_over_plain": value / plain_value}

    # --- voxel-boundary stepping against the reference's stepping, same medium and budgets ---
    if "exact_stepping" not in skip:
        sub = {}
        for label, ex in (("reference_stepping", 0), ("voxel_boundary_stepping", 1)):
            rx = mc.run_desc(EXC_PHOTONS // 10, det=m.det, photons_per_voxel=PHOTONS_PER_VOXEL // 10, fluence=1,
                             seed_exc=5 + 1000 * rank, seed_fl=6 + 1000 * rank, exact_stepping=ex)
            ox = mc.RunOut()
            mc.check(lib.mcfl_run(ctx.handle, med.handle, mc.ctypes.byref(rx), mc.ctypes.byref(ox)))  # warm-up
            mc.check(lib.mcfl_run(ctx.handle, med.handle, mc.ctypes.byref(rx), mc.ctypes.byref(ox)))
            sx, sfx = dict(zip(mc.STAT_NAMES, ox.stats_exc)), dict(zip(mc.STAT_NAMES, ox.stats_fl))
            sub[label] = {"photons_per_s": (rx.photons + ox.photons_fl) / ((ox.ms_exc + ox.ms_fl) / 1e3),
                          "excitation_photons": rx.photons, "emission_photons": ox.photons_fl,
                          "emitting_voxels": ox.fl_voxels, "passes_per_photon_exc": sx["steps"] / rx.photons,
                          "passes_per_photon_fl": sfx["steps"] / max(1, ox.photons_fl)}
        sub["workload"] = "the headline medium at a tenth of its budgets, fast math, two phases"
        result["exact_stepping"] = sub

    # --- batched sweep: 256 beams on the sphere medium ---
    if "batching" not in skip:
        c1 = media.config1()
        med1 = ctx.medium(c1.labels, c1.bulks, voxel_cm=c1.voxel_cm)
        scale = args.batching_scale
        pos, budgets = media.raster_sources(16, 4.0, seed=3, scale=scale)
        runs = [mc.run_desc(b, source=(x, y, 0.0), det=c1.det, seed_exc=10_000 + i) for i, ((x, y), b)
                in enumerate(zip(pos, budgets))]
        mc.batch_run(ctx, med1, runs[:4], mc.SCHEDULE_BATCHED, images=False)
        _, ms_b = mc.batch_run(ctx, med1, runs, mc.SCHEDULE_BATCHED, images=False)
        _, ms_p = mc.batch_run(ctx, med1, runs, mc.SCHEDULE_PLAIN, images=False)
        tot = sum(budgets)
        result["batching"] = {
            "workload": f"256 Gaussian beams on a 16x16 raster over the config-1 sphere medium (50^3 voxels, 4x4x2 cm), "
                        f"log-uniform budgets 1e6..5e7 scaled by {scale} ({tot:.3g} photons), own R/T images each",
            "batched_photons_per_s": tot / (ms_b / 1e3), "plain_photons_per_s": tot / (ms_p / 1e3),
            "batched_over_plain": ms_p / ms_b, "batched_ms": ms_b, "plain_ms": ms_p}
        # the same kind of sweep over several media in one launch (mixed-media kernel)
        c2 = media.config2(seed=2)
        med2 = ctx.medium(c2.labels, c2.bulks, voxel_cm=c2.voxel_cm, fluor_map=c2.fluor_map)
        c2b = media.config2(seed=7)
        med3 = ctx.medium(c2b.labels, c2b.bulks, voxel_cm=c2b.voxel_cm, fluor_map=c2b.fluor_map)
        pool = [med1, med2, med3]
        rng = np.random.default_rng(11)
        mruns, mmeds = [], []
        for i in range(96):
            k = i % 3
            b = int(np.exp(rng.uniform(np.log(1e5), np.log(5e6))))
            x, y = rng.uniform(-1.0, 1.0, 2)
            mruns.append(mc.run_desc(b, source=(float(x), float(y), 0.0), det=c1.det, seed_exc=20_000 + i))
            mmeds.append(pool[k])
        mc.batch_run(ctx, mmeds[:6], mruns[:6], mc.SCHEDULE_BATCHED, images=False)
        _, mb = mc.batch_run(ctx, mmeds, mruns, mc.SCHEDULE_BATCHED, images=False)
        _, mp = mc.batch_run(ctx, mmeds, mruns, mc.SCHEDULE_PLAIN, images=False)
        mt = sum(r.photons for r in mruns)
        result["batching"]["mixed_media"] = {
            "workload": f"96 Gaussian beams over 3 media (the sphere medium and two seeded config-2 media) in one "
                        f"launch, log-uniform budgets 1e5..5e6 ({mt:.3g} photons)",
            "batched_photons_per_s": mt / (mb / 1e3), "plain_photons_per_s": mt / (mp / 1e3),
            "batched_over_plain": mp / mb}
        med3.free()
        med2.free()
        med1.free()

    # --- continuous-batching server ---
    if "serving" not in skip:
        result["serving"] = serve_stream(mc, ctx, local, duration_s=12.0, express_period=args.express_period,
                                         express_ratio=args.express_ratio)

    # --- precision: the FP32 builds against the FP64 build on identical seeds ---
    if "precision" not in skip:
        result["precision"] = precision_section(mc, local, args.precision_photons)

    # --- CPU baseline (reference algorithm on host cores) ---
    if "cpu" not in skip:
        nthreads = os.cpu_count() or 1
        v, p, t, desc, ppp, phases = cpu_reference_sample(nthreads)
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": desc,
                                  "seconds": t, "passes_per_photon_exc": ppp, "phases": phases}
        # the same phases on the GPU, for the ratio of each phase alone
        result["cpu_baseline"]["gpu_over_cpu"] = {
            "excitation": result["phases"]["excitation_photons_per_s"] / phases["excitation_photons_per_s"]
            if phases.get("excitation_photons_per_s") else None,
            "emission": result["phases"]["emission_photons_per_s"] / phases["emission_photons_per_s"]
            if phases.get("emission_photons_per_s") else None}
    med.free()
    ctx.close()
    print(json.dumps(result), flush=True)
    if dist:
        torch.distributed.destroy_process_group()
    return 0


def precision_section(mc, device: int, photons: float, batches: int = 10):
    """The config-5 precision study at a bounded budget: 512 x 512 x 256
    voxels of 0.01 cm with a 268 MB fluorophore map, mu_s' = 20/cm, wide-field
    source; the fast-math and the exact-math FP32 builds and the FP64 build of
    the same kernel on the same seeds; integrated R, T and absorbed fraction
    (relative difference, paired z) and the R image against FP64."""
    from cudamcfl_gb300 import media, precision
    m = media.config5()
    ctx = mc.Context(device=device)
    try:
        med = ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
        w, h = m.info["widefield"]
        per_batch = int(photons) // batches

        def rd_for_seed(seed):
            return mc.run_desc(per_batch, det=m.det, fluence=0, seed_exc=seed, seed_fl=seed + 1,
                               kind=mc.SOURCE_WIDEFIELD, width=w, height=h)

        res = precision.study(ctx, med, rd_for_seed, batches, ("fast", "exact", "f64"), fluence=False)
        med.free()
    finally:
        ctx.close()
    out = precision.summarize(res)
    keep = {}
    for mode in ("fast", "exact"):
        o = out[mode]
        keep[mode] = {k: {q: o[k][q] for q in ("rel_diff", "paired_se_rel", "z")}
                      for k in ("R_total", "T_total", "absorbed")}
        keep[mode]["R_image"] = {q: o["R_image"].get(q) for q in ("entries", "rel_rms", "beyond_t", "t_threshold")}
        keep[mode]["passes_ratio"] = o["steps_ratio"]
    keep["photons_per_s"] = {k: v["photons_per_s"] for k, v in out["timing"].items()}
    keep["workload"] = (f"config5: 512x512x256 voxels of 0.01 cm (labels + 268 MB fp32 fluorophore map), "
                        f"mu_s' 20/cm, 5.12x5.12 cm wide-field source, {per_batch * batches:.3g} photons per build "
                        f"in {batches} batches on identical seeds; FP32 fast-math and exact-math builds vs the FP64 "
                        f"build of the same kernel (paired differences)")
    return keep


def profile_case(args):
    import cudamcfl_gb300 as mc
    from cudamcfl_gb300 import build, media
    build.build()
    ctx = mc.Context(device=0, math=mc.MATH_FAST if args.math == "fast" else mc.MATH_EXACT)
    ctx.set_option("variant", args.variant)
    ctx.set_option("pass_form", args.pass_form)
    ctx.set_option("phd_agg", args.phd_agg)
    if args.relaunch:
        ctx.set_option("relaunch", args.relaunch)
    m = media.config2(seed=2)
    med = ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
    rd = mc.run_desc(args.photons, det=m.det, photons_per_voxel=args.per_voxel, fluence=1, seed_exc=1, seed_fl=2,
                     exact_stepping=1 if args.exact_stepping else 0)
    best_exc = best_fl = float("inf")
    for _ in range(args.warmup + 1):
        r = ctx.run(med, rd, images=False, raw=False)
        best_exc, best_fl = min(best_exc, r.ms_exc), min(best_fl, r.ms_fl)
    print(json.dumps({"profile_case": "config2", "math": args.math, "photons": args.photons,
                      "exact_stepping": bool(args.exact_stepping),
                      "emission_photons": r.photons_fl, "steps_exc": r.stats_exc["steps"],
                      "steps_fl": r.stats_fl["steps"], "ms_exc": r.ms_exc, "ms_fl": r.ms_fl,
                      "best_ms_exc": best_exc, "best_ms_fl": best_fl,
                      "variant": args.variant, "pass_form": args.pass_form, "phd_agg": args.phd_agg,
                      "relaunch": ctx.get_option("relaunch"),
                      "regs": ctx.get_option("regs"),
                      "grid": ctx.get_option("grid"),
                      "block": ctx.get_option("launch_block")}), flush=True)
    med.free()
    ctx.close()
    return 0


def serve_stream(mc, ctx_main, device, duration_s: float = 12.0, seed: int = 4, express_period: int = 0,
                 express_ratio: int = 0, fifo: bool = True, saturated: bool = True):
    """Poisson arrivals at ~80 % of the measured service rate."""
    from cudamcfl_gb300 import media
    rng = np.random.default_rng(seed)
    sizes = [(64, 64, 64), (96, 96, 64), (128, 128, 64), (160, 160, 96), (192, 192, 128), (256, 256, 128)]
    pool = []
    for i, (nx, ny, nz) in enumerate(sizes):
        vox = (4.0 / nx, 4.0 / ny, 2.0 / nz)
        lab = np.ones((nz, ny, nx), dtype=np.uint8)
        fmap = np.zeros(lab.shape, dtype=np.float32)
        for j in range(int(rng.integers(2, 6))):
            media.add_sphere(lab, vox, (rng.uniform(-1.2, 1.2), rng.uniform(-1.2, 1.2), rng.uniform(0.4, 1.6)),
                             rng.uniform(0.15, 0.45), int(rng.integers(2, 4)), fmap, float(rng.uniform(0, 1)))
        bulks = [mc.outer_bulk(1.0), mc.bulk_from_mci_columns(1.4, 0.1, 100.0, g=0.9),
                 mc.bulk_from_mci_columns(1.4, 0.3, 80.0, 1.0, 0.05, 0.02, 0.1, 0.85),
                 mc.bulk_from_mci_columns(1.4, 0.05, 120.0, 1.0, 0.08, 0.03, 0.15, 0.9), mc.outer_bulk(1.0)]
        pool.append((lab, bulks, vox, fmap))
    det = mc.Detector(0.0, 0.0, 0.04, 0.04, 100, 100)
    # service rate from a calibration run (photons/s of a plain single run)
    lab, bulks, vox, fmap = pool[2]
    med = ctx_main.medium(lab, bulks, voxel_cm=vox, fluor_map=fmap)
    cal = ctx_main.run(med, mc.run_desc(5_000_000, det=det, seed_exc=9), images=False, raw=False)
    med.free()
    rate_photons = 5_000_000 / (cal.ms_exc / 1e3)
    mean_photons = (1e8 - 1e5) / math.log(1e8 / 1e5)
    lam = 0.8 * rate_photons / mean_photons
    import cudamcfl_gb300 as mcm
    sctx = mcm.Context(device=device, math=ctx_main.get_option("math"))
    policy = dict(express_period=express_period, express_ratio=express_ratio)
    srv = mcm.Server(sctx, max_jobs=64, **policy)
    ids, plain_ms_est = [], 0.0
    arrivals = []  # (offset s, pool index, run desc) to replay through a FIFO
    t_start = time.perf_counter()
    t_next = t_start
    n = 0
    while True:
        now = time.perf_counter()
        if now - t_start > duration_s:
            break
        if now < t_next:
            time.sleep(min(0.002, t_next - now))
            continue
        photons = int(math.exp(rng.uniform(math.log(1e5), math.log(1e8))))
        lab, bulks, vox, fmap = pool[int(rng.integers(0, len(pool)))]
        wide = rng.uniform() < 0.5
        rd = mcm.run_desc(photons, det=det, seed_exc=20_000 + n, kind=mcm.SOURCE_WIDEFIELD if wide else
                          mcm.SOURCE_GAUSS_BEAM, width=4.0, height=4.0, fluence=0)
        ids.append((srv.submit(lab, bulks, vox, rd, fluor_map=fmap), photons))
        arrivals.append((now - t_start, lab, bulks, vox, fmap, rd))
        n += 1
        t_next += rng.exponential(1.0 / lam)
    for rid, _ in ids:
        srv.wait(rid, -1)
    mtr = srv.metrics()
    served_lat = [srv.result(rid)["latency_ms"] for rid, _ in ids]
    sizes = [p for _, p in ids]
    srv.close()
    photons_total = sum(p for _, p in ids)
    served = photons_total / mtr["span_s"] if mtr["span_s"] > 0 else None
    out = {"requests": len(ids), "arrival_rate_per_s": lam, "target_load": 0.8, "p50_ms": mtr["p50_ms"],
           "p99_ms": mtr["p99_ms"], "max_ms": mtr["max_ms"], "mean_ms": float(np.mean(served_lat)),
           "photons_per_s": served, "express_period": express_period, "express_ratio": express_ratio,
           "mean_jobs_in_flight": mtr["mean_inflight"], "max_jobs_in_flight": mtr["max_inflight"],
           "slices": mtr["slices"], "server_busy_s": mtr["busy_s"], "server_upload_s": mtr["upload_s"],
           "server_finish_s": mtr["finish_s"], "server_kernel_s": mtr["kernel_s"], "server_span_s": mtr["span_s"],
           "workload": "Poisson requests at 80 % of the calibrated single-run rate, own media 64^3..256x256x128 "
                       "(labels + fp32 map), 1e5..1e8 photons log-uniform, Gaussian beam or 4x4 cm wide field; "
                       "saturated: 24 such requests queued at once vs run one per launch (upload, run, read back)"}
    out["slowest"] = {"served": sorted(((round(l, 1), p) for l, p in zip(served_lat, sizes)), reverse=True)[:4],
                      "note": "(latency ms, photons) of the four slowest requests"}

    if fifo:
        # the same arrivals through a FIFO that runs one request at a time
        # (upload, run, read back), the plain schedule a queue alone gives
        fifo_lat = []
        t0 = time.perf_counter()
        for off, lab, bulks, vox, fmap, rd in arrivals:
            now = time.perf_counter() - t0
            if now < off:
                time.sleep(off - now)
            med = sctx.medium(lab, bulks, voxel_cm=vox, fluor_map=fmap)
            sctx.run(med, rd, images=False, raw=True)
            med.free()
            fifo_lat.append(1e3 * (time.perf_counter() - t0 - off))
        fifo_span = time.perf_counter() - t0
        out["fifo"] = {"p50_ms": float(np.percentile(fifo_lat, 50)), "p99_ms": float(np.percentile(fifo_lat, 99)),
                       "mean_ms": float(np.mean(fifo_lat)),
                       "max_ms": float(np.max(fifo_lat)), "photons_per_s": photons_total / fifo_span,
                       "note": "the same arrivals, one request at a time in arrival order"}
        out["slowest"]["fifo"] = sorted(((round(l, 1), p) for l, p in zip(fifo_lat, sizes)), reverse=True)[:4]

    if saturated:
        # saturation: the same kind of requests all queued at once (served),
        # and one request per launch after another (plain), same requests;
        # a generator of their own, so that every run draws the same 24
        brng = np.random.default_rng(seed + 1000)
        burst = []
        for i in range(24):
            photons = int(math.exp(brng.uniform(math.log(1e5), math.log(1e8))))
            lab, bulks, vox, fmap = pool[int(brng.integers(0, len(pool)))]
            wide = brng.uniform() < 0.5
            burst.append((lab, bulks, vox, fmap, mcm.run_desc(photons, det=det, seed_exc=90_000 + i, width=4.0,
                                                             height=4.0, kind=mcm.SOURCE_WIDEFIELD if wide else
                                                             mcm.SOURCE_GAUSS_BEAM)))
        srv = mcm.Server(sctx, max_jobs=64, **policy)
        t0 = time.perf_counter()
        bids = [srv.submit(lab, bulks, vox, rd, fluor_map=fmap) for lab, bulks, vox, fmap, rd in burst]
        for rid in bids:
            srv.wait(rid, -1)
        t_served = time.perf_counter() - t0
        for rid in bids:
            srv.result(rid)
        srv.close()
        t0 = time.perf_counter()
        for lab, bulks, vox, fmap, rd in burst:
            med = sctx.medium(lab, bulks, voxel_cm=vox, fluor_map=fmap)
            sctx.run(med, rd, images=False, raw=True)
            med.free()
        t_plain = time.perf_counter() - t0
        burst_photons = sum(b[4].photons for b in burst)
        out["saturated"] = {"requests": len(burst), "photons": burst_photons,
                            "served_photons_per_s": burst_photons / t_served,
                            "plain_photons_per_s": burst_photons / t_plain, "served_over_plain": t_plain / t_served}
    sctx.close()
    return out

if __name__ == "__main__":
    sys.exit(main())
