#!/usr/bin/env python
"""Benchmark of the fluid step: PBF particle-steps/s on the 1,048,576-particle
double dam break, iterating every step until the mean one-sided density error
is <= 0.1 %, with the learned warm start (the headline `value`) and with the
plain method beside it (config.plain).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

One JSON line on rank 0.  Timing: every timed step is bracketed by CUDA events
on the stream the step is enqueued on, with a 256 MiB L2 flush between steps
(outside the events); max over ranks; W >= 3 untimed warm-up steps after a
100-step pre-roll that brings the dam break into its collapsing phase.
Multi-GPU runs are independent replicas (the path does not shard; weak scaling).

Legs of the line:
  value / ms_per_step  device-resident steps, learned warm start (graph launch per step)
  config.plain         the same window with the plain method (no warm start)
  e2e                  the warm-start steps through the public API with the whole
                       particle state crossing host<->device every step (pinned buffers)
  roofline             the dominant kernel, algorithmic bytes per launch over its
                       event-timed duration, against MEASURED_PEAKS.json
  cpu_baseline         the reference's own CPU code (oracle/_ref; the oracle
                       restatement when unavailable) on a bounded sample
--impl reference prints the reference CPU arm alone.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PBF particle-steps/s at 1M, learned warm-start vs plain, at 0.1% density error"
UNIT = "particle-steps/s"
WORKLOAD = "pbf_double_dam_break_1M"
BLOCK = (64, 64, 128)
PREROLL = 100
# constraint iterations per step of the reference CPU arm (its loop is run with
# eta = 0, i.e. exactly this many): the plain GPU method's mean over the timed
# window of this workload (steps 104-123 after the pre-roll), 55.65 measured
REF_ITERS = 56
REF_BLOCK = (12, 12, 24)
# algorithmic (compulsory) bytes per particle of one launch
BYTES_LAMBDA = 24.0       # R x* 16, W lambda 4, W rho 4
BYTES_CORRECTION = 36.0   # R x* 16, R lambda 4, W x* 16


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def replica_rate(units_per_rank: int, steps: int, secs: float, dist=None):
    """Whole-job rate of independent replicas: every rank processed
    units_per_rank x steps units; the job took the slowest rank's time.
    Returns (units/s over all ranks, that time in seconds)."""
    world = 1
    if dist is not None:
        import torch
        t = torch.tensor([secs], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        secs = float(t.item())
        world = dist.get_world_size()
    return units_per_rank * steps * world / secs, secs


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def method_of(meta: dict) -> str:
    """The warm-start method as the bench line names it."""
    local = ", 16 local inputs weighted" if meta.get("features") == "base" else ""
    return f"learned warm start (BF16 MLP 32-64-64-3{local})"


def make_scene(block=BLOCK, warm_start=0):
    from fltk_sph_ice_gb300 import abi, scenes
    sc = scenes.pbf_double_dam_break(block=block)
    p = sc.params
    p.eta = 1e-3
    p.error_mode = abi.ERR_ONE_SIDED
    p.clamp_constraint = 1
    p.min_iter = 2
    p.max_iter = 400
    p.use_graph = 1
    p.warm_start = warm_start
    # list skin 0.1 h: with ~11 warm-started iterations per step one grid
    # build per step beats shorter lists (measured: 2.90 ms per step against
    # 2.97 at 0.05, 3.00 at 0.07, 3.09 at 0.04)
    p.cell_skin = 0.1
    return sc


# ---------------------------------------------------------------------------
# CPU: the reference's own code (oracle/_ref) or the oracle restatement
# ---------------------------------------------------------------------------
def cpu_sample(pos, vel, params, iters: int, steps: int = 1):
    """Seconds per step of the reference CPU PBF Update on this state, with
    the loop fixed at `iters` iterations (eta = 0), on one host thread."""
    import oracle
    from fltk_sph_ice_gb300 import abi
    p = abi.FsphParams.from_buffer_copy(params)
    p.eta, p.min_iter, p.max_iter = 0.0, min(2, iters), iters
    p.error_mode = abi.ERR_TWO_SIDED
    n = pos.shape[0]
    kind = "reference"
    try:
        s = oracle.RefSolver(p, n, "pbf")
    except RuntimeError:
        kind = "port"
        s = oracle.Oracle(p, n, "float", threads=1)
    s.set(pos, vel)
    t0 = time.perf_counter()
    for _ in range(steps):
        if kind == "reference":
            s.update(float(0.0016))
        else:
            s.pbf_step(0.0016, fixed_iters=iters)
    dt = (time.perf_counter() - t0) / steps
    return dt, kind


def cpu_sample_state(preroll: int = PREROLL, threads: int = 0):
    """The CPU legs' sample: the REF_BLOCK double dam break with the GPU arms'
    constants (unilateral constraint, iterate to 0.1 %, XSPH, vorticity)
    after `preroll` steps, stepped by the FP32 oracle on the host cores.  The
    cpu_baseline leg and the reference arm both time the reference's step on
    this one state.  Returns (scene, positions, velocities)."""
    import oracle
    sc = make_scene(REF_BLOCK)
    o = oracle.Oracle(sc.params, sc.n, "float", threads=threads or host_cores())
    o.set(sc.pos, sc.vel)
    for _ in range(preroll):
        o.pbf_step(sc.dt)
    return sc, o.get("pos"), o.get("vel")


def _reference_worker(job):
    """One host core: warm-up + timed steps of the reference CPU Update on
    its own copy of the sample state; returns (seconds per timed step, kind)."""
    warmup, steps, pos, vel, iters = job
    sc = make_scene(REF_BLOCK)
    kind = "reference"
    for _ in range(warmup):
        cpu_sample(pos, vel, sc.params, iters)
    times = []
    for _ in range(steps):
        t, kind = cpu_sample(pos, vel, sc.params, iters)
        times.append(t)
    return times, kind


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_arm(args):
    """The reference's CPU PBF step on every host core: one process per core,
    each stepping its own copy of the sample scene; the aggregate rate is all
    particle-steps over the slowest process's time."""
    import multiprocessing as mp
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    cores = host_cores()
    sc, xs, vs = cpu_sample_state(args.preroll)
    n = sc.n
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_reference_worker, [(max(args.warmup, 0), args.steps, xs, vs, REF_ITERS)] * cores)
    kind = res[0][1]
    tot = max(sum(t) for t, _ in res)
    value = cores * n * args.steps / tot
    sample = (f"one PBF step of the {n}-particle double dam break (blocks {REF_BLOCK[0]}x{REF_BLOCK[1]}x"
              f"{REF_BLOCK[2]}) after a {args.preroll}-step pre-roll (FP32 oracle, the GPU arms' constants), "
              f"the same state as the GPU line's cpu_baseline, per timed step and process; {REF_ITERS} fixed "
              f"constraint iterations (the plain GPU method's mean on the 1M window); {cores} processes, one "
              f"per host core")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "sample_particles": n, "iterations": REF_ITERS,
                                        "processes": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_leg(ctx, warm: bool, blob):
    """Pre-roll, warm up and time args.steps steps of one method; returns the
    context (kept alive for the later legs) and the per-step record."""
    torch, L, abi, args, stream, flush, dist = (ctx[k] for k in ("torch", "L", "abi", "args", "stream", "flush",
                                                                  "dist"))
    from fltk_sph_ice_gb300 import rxPBDSPH
    sc = make_scene(warm_start=1 if warm else 0)
    if args.eager:
        sc.params.use_graph = 0
    ps = rxPBDSPH(sc.params)
    if warm:
        st = L.fsph_set_warm_start_model(ps.handle, blob.ctypes.data_as(ctypes.c_void_p))
        if st != abi.OK:
            raise abi.FsphError(st, "fsph_set_warm_start_model")
    ps.Set(sc.pos, sc.vel)
    sp = ctypes.c_void_p(stream.cuda_stream)
    stats = abi.FsphStepStats()

    def step():
        st = L.fsph_step(ps.handle, ctypes.c_float(sc.dt), sp, None)
        if st != abi.OK:
            raise abi.FsphError(st, L.fsph_last_error(ps.handle).decode())

    for _ in range(args.preroll + max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    iters, errs, kernels, builds, unconv = [], [], [], [], 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
        stream.synchronize()
        L.fsph_last_stats(ps.handle, ctypes.byref(stats))
        iters.append(stats.iterations)
        errs.append(stats.density_error_one_sided)
        kernels.append(stats.kernels)
        builds.append(stats.grid_builds)
        unconv += int(stats.status == abi.NOT_CONVERGED)
    torch.cuda.synchronize()
    tot_ms = sum(a.elapsed_time(b) for a, b in ev)
    n = sc.n
    value, secs = replica_rate(n, args.steps, tot_ms / 1000.0, dist)
    tot_ms = secs * 1000.0
    return ps, sc, {"value": value, "ms_per_step": tot_ms / args.steps,
                    "mean_iterations": float(np.mean(iters)), "max_error": float(np.max(errs)),
                    "iterations": iters, "kernels": int(sum(kernels)), "grid_builds": float(np.mean(builds)),
                    "not_converged_steps": unconv, "status": "FSPH_NOT_CONVERGED" if unconv else "FSPH_OK"}


TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "k_lambda_k_correction_pbf_double_dam_break_1M.md")
# the sources of the constraint-pass kernels: a profile's figures hold for the
# kernels built from exactly these files
KERNEL_SOURCES = ("fltk_sph_ice_gb300/csrc/fsph_passes.cuh", "fltk_sph_ice_gb300/csrc/fsph_kernels.cu",
                  "fltk_sph_ice_gb300/csrc/fsph_kernels.cuh", "fltk_sph_ice_gb300/csrc/fsph_internal.cuh")


def kernel_sources_digest() -> str:
    """sha256 (first 12 hex digits) of the constraint-pass kernel sources."""
    import hashlib
    h = hashlib.sha256()
    for rel in KERNEL_SOURCES:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:12]


def profile_digest():
    """The kernel-sources digest the committed profile was captured at (its
    'Kernel sources digest' line), or None."""
    import re
    if not os.path.isfile(TRAFFIC_PROFILE):
        return None
    with open(TRAFFIC_PROFILE) as f:
        m = re.search(r"Kernel sources digest: `([0-9a-f]+)`", f.read())
    return m.group(1) if m else None


def profile_current() -> bool:
    """The committed profile describes the kernels of this build."""
    d = profile_digest()
    return d is not None and d == kernel_sources_digest()


def ncu_traffic(kname: str):
    """DRAM bytes (read + write) of one launch of kname at 1M particles, from
    the committed ncu summary's 'traffic per launch' row (its first two
    columns are the current kernels); None if absent or captured from other
    kernel sources than these."""
    import re
    if not profile_current():
        return None
    with open(TRAFFIC_PROFILE) as f:
        for line in f:
            if line.startswith("| **traffic per launch**"):
                mb = [float(x) for x in re.findall(r"([0-9.]+) MB", line)]
                col = {"k_lambda": 0, "k_correction": 1}.get(kname)
                if col is not None and len(mb) >= 2:
                    return mb[col] * 1e6
    return None


def ncu_warp_instructions(kname: str):
    """Warp instructions of one launch of kname at 1M particles, from the
    committed ncu summary's 'warp instructions' row; None if absent or
    captured from other kernel sources than these."""
    import re
    if not profile_current():
        return None
    with open(TRAFFIC_PROFILE) as f:
        for line in f:
            if line.startswith("| warp instructions"):
                m = [float(x) for x in re.findall(r"([0-9.]+) M", line)]
                col = {"k_lambda": 0, "k_correction": 1}.get(kname)
                if col is not None and len(m) >= 2:
                    return m[col] * 1e6
    return None


def ncu_l1tex(kname: str):
    """L1TEX throughput of one launch of kname at 1M particles, % of its peak
    while the SMs are active, from the committed ncu summary (the pass's
    binding unit: the gathered positions and streamed list groups); None if
    absent or captured from other kernel sources than these."""
    import re
    if not profile_current():
        return None
    with open(TRAFFIC_PROFILE) as f:
        for line in f:
            if line.startswith("| **L1TEX throughput"):
                m = [float(x) for x in re.findall(r"([0-9.]+) %", line)]
                col = {"k_lambda": 0, "k_correction": 1}.get(kname)
                if col is not None and len(m) >= 2:
                    return {"pct_of_peak_active": m[col], "source": "ncu l1tex__throughput"}
    return None


def issue_bound(kname: str, launch_ms: float):
    """The pass against the instruction-issue bound: the profiled warp
    instructions of one launch over its live launch time, against one warp
    instruction per SM sub-partition per clock (152 SMs x 4 at the maximum
    SM clock of MEASURED_PEAKS.json, else 2070 MHz); None without a profile."""
    try:
        inst = ncu_warp_instructions(kname)
        if inst is None or not launch_ms > 0:
            return None
        mhz = 2070.0
        p = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.isfile(p):
            with open(p) as f:
                mhz = float(json.load(f).get("sm_max_mhz", mhz))
        peak = 152 * 4 * mhz * 1e6 / 1e12
        achieved = inst / (launch_ms / 1000.0) / 1e12
        return {"unit": "T warp instructions/s", "warp_instructions": inst, "achieved": achieved, "peak": peak,
                "frac": achieved / peak}
    except (OSError, ValueError, TypeError):
        return None


def roofline_of(L, abi, ps, n, mean_iters):
    t_lam, t_cor, t_grid, t_list = (ctypes.c_float(0) for _ in range(4))
    L.fsph_time_pass(ps.handle, abi.PASS_LAMBDA, 20, ctypes.byref(t_lam))
    L.fsph_time_pass(ps.handle, abi.PASS_CORRECTION, 20, ctypes.byref(t_cor))
    L.fsph_time_pass(ps.handle, abi.PASS_GRID, 10, ctypes.byref(t_grid))
    L.fsph_time_pass(ps.handle, abi.PASS_LIST, 10, ctypes.byref(t_list))
    if t_cor.value >= t_lam.value:
        kname, kms, kbytes = "k_correction", t_cor.value, BYTES_CORRECTION * n
    else:
        kname, kms, kbytes = "k_lambda", t_lam.value, BYTES_LAMBDA * n
    peak, peak_kind = measured_peaks()
    achieved = kbytes / (kms / 1000.0) / 1e9
    traffic = ncu_traffic(kname)
    digest = kernel_sources_digest()
    src = (f"ncu, profiles/{os.path.basename(TRAFFIC_PROFILE)} (kernel sources {digest})" if profile_current()
           else f"none: the committed profile was captured from other kernel sources than these ({digest})")
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "traffic_source": src, "kernel": kname, "launch_ms": kms, "peak_kind": peak_kind,
            "lambda_ms": t_lam.value, "correction_ms": t_cor.value, "grid_build_ms": t_grid.value,
            "list_build_ms": t_list.value, "issue": issue_bound(kname, kms), "l1tex": ncu_l1tex(kname),
            "passes_ms_per_step": mean_iters * (t_lam.value + t_cor.value)}


# compulsory HBM bytes per particle-step of a PBF step with I constraint
# iterations: B(I) = 396 + 60 I (prediction 48, one grid build 120, 60 per
# iteration, finalize / XSPH / vorticity 228); the learned warm start adds its
# network inputs (16 floats read, 64 B) and the predicted correction (16 B)
def step_bytes(iters: float, warm_start: bool = False) -> float:
    return 396.0 + 60.0 * iters + (80.0 if warm_start else 0.0)


def step_roofline(value: float, iters: float, builds: float, warm_start: bool = False):
    """The whole step against HBM: compulsory bytes per particle-step x
    particle-steps/s.  In-loop grid rebuilds (builds - 1 per step) are the
    implementation's choice and are not counted."""
    peak, peak_kind = measured_peaks()
    b = step_bytes(iters, warm_start)
    achieved = value * b / 1e9
    return {"bytes_per_particle_step": b, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind, "iterations": iters, "grid_builds": builds}


FP64_REPLICA = (12, 12, 24)
FP64_STEPS = 20
FP64_ITERS = 10


def fp64_error_headline(abi, rxPBDSPH):
    """FP32 GPU against the FP64 oracle, step by step, on a 6,912-particle
    replica of the headline scene (same constants: unilateral constraint,
    XSPH, vorticity), both with a fixed iteration count so the two runs do
    the same work: max |x_gpu - x_fp64| / h per step, and the density error
    of the last step's lambda pass."""
    import oracle
    sc = make_scene(FP64_REPLICA)
    p = sc.params
    p.min_iter = p.max_iter = FP64_ITERS
    p.eta = 0.0
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    o = oracle.Oracle(p, sc.n, precision="double", threads=host_cores())
    o.set(sc.pos, sc.vel)
    out = []
    for _ in range(FP64_STEPS):
        ps.Update(sc.dt)
        o.pbf_step(sc.dt, fixed_iters=FP64_ITERS)
        d = ps.GetArrayVBO(abi.RX_POSITION)[:, :3].astype(np.float64) - o.get("pos")[:, :3]
        out.append(float(np.abs(d).max() / p.h))
    rho = ps.GetArrayVBO(abi.RX_DENSITY).astype(np.float64)
    rho64 = o.get("dens").astype(np.float64)
    ps.close()
    return {"replica_particles": sc.n, "iterations": FP64_ITERS, "max_abs_position_error_over_h": out,
            "last_step_density_max_rel_error": float(np.abs(rho - rho64).max() / np.abs(rho64).max())}


def e2e_leg(ctx, ps, sc):
    """The public API with host buffers: the whole particle state goes host ->
    device (SetArrayVBO) and back (GetArrayVBO) around every step."""
    torch, L, abi, args, dist = (ctx[k] for k in ("torch", "L", "abi", "args", "dist"))
    n = sc.n
    pin_pos = torch.from_numpy(ps.GetArrayVBO(abi.RX_POSITION)).pin_memory().numpy()
    pin_vel = torch.from_numpy(ps.GetArrayVBO(abi.RX_VELOCITY)).pin_memory().numpy()
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731

    def e2e_step():
        st = L.fsph_set_array(ps.handle, abi.RX_POSITION, vp(pin_pos), 0, n, abi.HOST)
        st |= L.fsph_set_array(ps.handle, abi.RX_VELOCITY, vp(pin_vel), 0, n, abi.HOST)
        st |= L.fsph_step(ps.handle, ctypes.c_float(sc.dt), None, None)
        st |= L.fsph_get_array(ps.handle, abi.RX_POSITION, vp(pin_pos), abi.HOST, None)
        st |= L.fsph_get_array(ps.handle, abi.RX_VELOCITY, vp(pin_vel), abi.HOST, None)
        if st != abi.OK:
            raise abi.FsphError(st, L.fsph_last_error(ps.handle).decode())

    for _ in range(3):
        e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    secs = time.perf_counter() - t0
    value, _ = replica_rate(n, args.steps, secs, dist)
    return {"value": value, "unit": UNIT, "h2d_bytes_per_step": 2 * 16 * n, "d2h_bytes_per_step": 2 * 16 * n}


def gpu_arm(args):
    import torch
    from fltk_sph_ice_gb300 import abi, build, rxPBDSPH, warmstart

    rank, world, local = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    build.build()
    L = abi.lib()
    blob, meta = warmstart.load_model(args.model)
    ctx = {"torch": torch, "L": L, "abi": abi, "args": args, "stream": torch.cuda.Stream(), "dist": dist,
           "world": world, "flush": torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")}

    with ClockSampler(local) as clk:
        ps_p, sc, plain = run_leg(ctx, False, blob) if not args.no_plain else (None, None, None)
        if ps_p is not None:
            ps_p.close()
        ps, sc, warm = run_leg(ctx, True, blob)
    clocks = clk.summary()
    n = sc.n
    roofline = roofline_of(L, abi, ps, n, warm["mean_iterations"])
    # the passes above advanced the state; a fresh warm-start context for e2e
    ps.close()
    e2e = None
    if not args.no_e2e:
        ps2, sc2, _ = run_leg(dict(ctx, args=argparse.Namespace(**{**vars(args), "steps": 1})), True, blob)
        e2e = e2e_leg(ctx, ps2, sc2)
        ps2.close()

    cpu = None
    fp64 = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sm, xs, vs = cpu_sample_state(args.preroll)
        ci = max(1, int(round(plain["mean_iterations"] if plain else REF_ITERS)))
        secs, kind = cpu_sample(xs, vs, sm.params, ci)
        cpu = {"value": sm.n / secs, "unit": UNIT, "cores": 1, "kind": kind,
               "sample": (f"one PBF step of the {sm.n}-particle double dam break (blocks {REF_BLOCK[0]}x"
                          f"{REF_BLOCK[1]}x{REF_BLOCK[2]}) after a {args.preroll}-step pre-roll (FP32 oracle, the "
                          f"GPU arms' constants; the reference arm times the same state), {ci} fixed constraint "
                          f"iterations (the plain GPU mean on the 1M window), 1 host thread"),
               "gpu_warm_over_cpu": warm["value"] / (sm.n / secs)}
        if plain:
            cpu["gpu_plain_over_cpu"] = plain["value"] / (sm.n / secs)
        fp64 = fp64_error_headline(abi, rxPBDSPH)

    # kernel launches of the timed warm-start steps, counted by the library from the step graph's
    # kernel nodes, the executed iterations and the grid rebuilds (eager mode does not count them:
    # MLP, predict+hash, 3 scan, scatter, cell sort, gather, list build, 2 per iteration, finalize,
    # XSPH/vorticity/features, vorticity apply, without rebuilds)
    gpu_launches = warm["kernels"] or int(args.steps * (12 + 2 * warm["mean_iterations"]))
    if rank == 0:
        cfg = {"workload": WORKLOAD, "particles": n, "block": list(BLOCK), "dt": sc.dt, "eta_one_sided": 1e-3,
               "constraint": "unilateral (clamped C >= 0)", "method": method_of(meta),
               "mean_iterations": warm["mean_iterations"], "max_error": warm["max_error"],
               "not_converged_steps": warm["not_converged_steps"], "status": warm["status"],
               "meets_criterion": warm["not_converged_steps"] == 0,
               "grid_builds_per_step": warm["grid_builds"], "cell_skin": round(float(sc.params.cell_skin), 3),
               "model": {"samples": meta.get("samples"), "rollouts": meta.get("rollouts"),
                         "output_damping": meta.get("output_damping")},
               "preroll_steps": args.preroll, "l2": "256 MiB flush between timed steps",
               "parallelism": f"replicas x{world}", "fp64_error_per_step": fp64}
        if plain:
            cfg["plain"] = {k: plain[k] for k in ("value", "ms_per_step", "mean_iterations", "max_error",
                                                  "grid_builds")}
            cfg["speedup_vs_plain"] = warm["value"] / plain["value"]
            roofline["step_plain"] = step_roofline(plain["value"], plain["mean_iterations"],
                                                   plain["grid_builds"])
        roofline["step_warm"] = step_roofline(warm["value"], warm["mean_iterations"], warm["grid_builds"],
                                              warm_start=True)
        line = {
            "metric": METRIC, "value": warm["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": warm["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattices)",
            "config": cfg, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": gpu_launches,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


C2_METRIC = "PBF particle-steps/s, 262,144-particle dam break, 4 constraint iterations"
C1_METRIC = "WCSPH particle-steps/s, 32,768-particle dam break"
CONFIG_PREROLL = 100
# compulsory HBM bytes per particle-step of a WCSPH step: one grid build 120,
# density pass 24 (R x, W rho, W p), force pass 56 (R x, v, rho, p, W a),
# integrate 80 (R x, v, a, W x, v)
WCSPH_BYTES = 120.0 + 24.0 + 56.0 + 80.0


def config_arm(args):
    """The 262,144-particle PBF dam break (4 fixed iterations, XSPH,
    vorticity) or the 32,768-particle WCSPH dam break, device-resident steps
    after a pre-roll; e2e through the public API with host buffers; the
    reference's CPU step on the same state (one host thread) as cpu_baseline."""
    import torch
    from fltk_sph_ice_gb300 import abi, build, rxPBDSPH, rxSPH, scenes

    rank, world, local = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    build.build()
    L = abi.lib()
    pbf = args.workload == "pbf_dam_break_262k"
    if pbf:
        sc = scenes.pbf_dam_break(64)
        p = sc.params
        p.eta, p.min_iter, p.max_iter = 0.0, 4, 4
        cls, metric = rxPBDSPH, C2_METRIC
    else:
        sc = scenes.wcsph_dam_break(32)
        p = sc.params
        cls, metric = rxSPH, C1_METRIC
    if args.eager:
        p.use_graph = 0
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ps = cls(p)
    ps.Set(sc.pos, sc.vel)

    def step():
        st = L.fsph_step(ps.handle, ctypes.c_float(sc.dt), sp, None)
        if st != abi.OK:
            raise abi.FsphError(st, L.fsph_last_error(ps.handle).decode())

    for _ in range(CONFIG_PREROLL):
        step()
    torch.cuda.synchronize()
    x0, v0 = ps.GetArrayVBO(abi.RX_POSITION), ps.GetArrayVBO(abi.RX_VELOCITY)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = abi.FsphStepStats()
    kern, builds = 0, []
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
            stream.synchronize()
            L.fsph_last_stats(ps.handle, ctypes.byref(stats))
            kern += stats.kernels
            builds.append(stats.grid_builds)
        torch.cuda.synchronize()
    tot_s = sum(a.elapsed_time(c) for a, c in ev) / 1000.0
    value, tot_s = replica_rate(sc.n, args.steps, tot_s, dist)
    peak, peak_kind = measured_peaks()
    if pbf:
        roof = roofline_of(L, abi, ps, sc.n, 4.0)
        roof["step"] = step_roofline(value, 4.0, float(np.mean(builds)))
    else:
        roof = sph_roofline(L, abi, ps, sc.n)
        b = WCSPH_BYTES
        roof["step"] = {"bytes_per_particle_step": b, "achieved": value * b / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": value * b / 1e9 / peak, "peak_kind": peak_kind}
    e2e = None
    if not args.no_e2e:
        e2e = e2e_leg({"torch": torch, "L": L, "abi": abi, "args": args, "dist": dist}, ps, sc)
    ps.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        import oracle
        nsteps = 1 if pbf else 5
        kind = "reference"
        try:
            r = oracle.RefSolver(p, sc.n, "pbf" if pbf else "sph")
        except RuntimeError:
            kind = "port"
            r = oracle.Oracle(p, sc.n, "float", threads=1)
        r.set(x0, v0)
        t0 = time.perf_counter()
        for _ in range(nsteps):
            if kind == "reference":
                r.update(float(sc.dt))
            elif pbf:
                r.pbf_step(sc.dt, fixed_iters=4)
            else:
                r.sph_step(sc.dt)
        secs = (time.perf_counter() - t0) / nsteps
        cpu = {"value": sc.n / secs, "unit": UNIT, "cores": 1, "kind": kind,
               "sample": (f"{nsteps} step(s) of the same {sc.n}-particle scene from the GPU's state after its "
                          f"{CONFIG_PREROLL}-step pre-roll, 1 host thread"
                          + (" (the reference's own loop fixed at 4 iterations; no XSPH / vorticity, which its "
                             "CPU path lacks)" if pbf else "")),
               "gpu_over_cpu": value / (sc.n / secs)}
    if rank == 0:
        line = {
            "metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1000.0 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": args.workload, "particles": sc.n, "dt": sc.dt, "preroll_steps": CONFIG_PREROLL,
                       "iterations": 4 if pbf else None, "grid_builds_per_step": float(np.mean(builds)),
                       "l2": "256 MiB flush between timed steps", "parallelism": f"replicas x{world}"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": kern or None,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def sph_roofline(L, abi, ps, n):
    """The WCSPH density and force passes, each timed alone (20 launches,
    CUDA events), against HBM with their compulsory bytes (24 and 56 B per
    particle)."""
    t_d, t_f = ctypes.c_float(0), ctypes.c_float(0)
    L.fsph_time_pass(ps.handle, abi.PASS_SPH_DENSITY, 20, ctypes.byref(t_d))
    L.fsph_time_pass(ps.handle, abi.PASS_SPH_FORCE, 20, ctypes.byref(t_f))
    peak, peak_kind = measured_peaks()
    if t_f.value >= t_d.value:
        kname, kms, kb = "k_sph_force", t_f.value, 56.0 * n
    else:
        kname, kms, kb = "k_sph_density", t_d.value, 24.0 * n
    achieved = kb / (kms / 1000.0) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": kname, "launch_ms": kms, "peak_kind": peak_kind,
            "density_ms": t_d.value, "force_ms": t_f.value}


BATCH_METRIC = "PBF particle-steps/s, 256 batched scenes of 2k-66k particles, 4 constraint iterations"
BATCH_PREROLL = 10
BATCH_ITERS = 4
# compulsory HBM bytes per particle-step of a 4-iteration step, B(I) = 396 + 60 I
BATCH_BYTES = 396.0 + 60.0 * BATCH_ITERS


def batched_arm(args):
    """The batched-scenes workload: every scene of the seeded 256-scene set
    steps together (one persistent launch per pass, the step one CUDA graph),
    launch shape from the library's autotuner.  One JSON line on rank 0."""
    import torch
    from fltk_sph_ice_gb300 import PBFBatch, abi, build, scenes

    rank, world, local = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    build.build()
    sc = scenes.batched_scenes()
    for s in sc:
        s.params.min_iter = BATCH_ITERS
        s.params.max_iter = BATCH_ITERS
    pos = np.concatenate([s.pos for s in sc])
    vel = np.concatenate([s.vel for s in sc])
    b = PBFBatch([s.params for s in sc], [s.n for s in sc], iterations=BATCH_ITERS)
    b.set_particles(pos, vel)
    n, dt = b.n, sc[0].dt
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(BATCH_PREROLL):
        b.step(dt, sp)
    if args.no_tune:  # the default configuration (256 threads, 1 lane, skin 0.05)
        cfg, tune_ms = b.config, None
    else:
        cfg, tune_ms = b.autotune(dt, steps=3)
    if args.eager:  # the same kernels with the loop on the host (profilers)
        b.set_config(cfg.block, cfg.lanes, cfg.cell_skin, eager=True)
    for _ in range(max(args.warmup, 3)):
        b.step(dt, sp)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev[k][0].record(stream)
            b.step(dt, sp)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    tot_s = sum(a.elapsed_time(c) for a, c in ev) / 1000.0
    value, tot_s = replica_rate(n, args.steps, tot_s, dist)
    errs = [b.scene_stats(s) for s in range(b.nscenes)]
    e2e_value = None
    if not args.no_e2e:
        # e2e: the whole batch host -> device, one step, positions and velocities back
        x_h = torch.from_numpy(b.get(abi.RX_POSITION)).pin_memory().numpy()
        v_h = torch.from_numpy(b.get(abi.RX_VELOCITY)).pin_memory().numpy()
        for _ in range(2):
            b.set_particles(x_h, v_h)
            b.step(dt)
            x_h[:] = b.get(abi.RX_POSITION)
            v_h[:] = b.get(abi.RX_VELOCITY)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            b.set_particles(x_h, v_h)
            b.step(dt)
            x_h[:] = b.get(abi.RX_POSITION)
            v_h[:] = b.get(abi.RX_VELOCITY)
        e2e_value, _ = replica_rate(n, args.steps, time.perf_counter() - t0, dist)
    peak, peak_kind = measured_peaks()
    achieved = value * BATCH_BYTES / 1e9
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        small = min(sc, key=lambda s: s.n)
        secs, kind = cpu_sample(small.pos, small.vel, small.params, BATCH_ITERS)
        cpu = {"value": small.n / secs, "unit": UNIT, "cores": 1, "kind": kind,
               "sample": f"one 4-iteration PBF step of the smallest batched scene ({small.n} particles), "
                         f"1 host thread"}
    if rank == 0:
        line = {
            "metric": BATCH_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1000.0 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattices)",
            "config": {"workload": "batched_256", "scenes": b.nscenes, "particles": n,
                       "iterations": BATCH_ITERS, "preroll_steps": BATCH_PREROLL,
                       "autotuned": {"block": cfg.block, "lanes": cfg.lanes, "cell_skin": round(cfg.cell_skin, 3),
                                     "ms_per_step_at_tuning": tune_ms},
                       "mean_error_one_sided": float(np.mean([e.density_error_one_sided for e in errs])),
                       "l2": "256 MiB flush between timed steps", "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "kernel": "whole step",
                         "bytes_per_particle_step": BATCH_BYTES, "peak_kind": peak_kind},
            "cpu_baseline": cpu,
            "e2e": None if e2e_value is None else {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n,
                                                   "d2h_bytes_per_step": 32 * n},
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    b.close()
    if dist:
        dist.destroy_process_group()
    return 0


LARGE_METRIC = ("PBF particle-steps/s at 16.8M particles with a boundary obstacle, learned warm start, "
                "0.1% density error")
LARGE_PREROLL = 10
LARGE_REPLICA = 16       # lattice side of the replica the FP64 oracle follows step by step
LARGE_REPLICA_STEPS = 20
LARGE_REPLICA_ITERS = 10


def fp64_error_per_step(abi, rxPBDSPH, scenes):
    """FP32 GPU (compensated density) against the FP64 oracle, step by step,
    on a small replica of the obstacle scene, both with a fixed iteration
    count: max |x_gpu - x_fp64| / h per step."""
    import oracle
    sc = scenes.pbf_obstacle_drop(n_side=LARGE_REPLICA)
    p = sc.params
    p.min_iter = p.max_iter = LARGE_REPLICA_ITERS
    p.compensated_density = 1
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    ps.SetBoundary(sc.boundary)
    o = oracle.Oracle(p, sc.n, precision="double", threads=host_cores())
    o.set(sc.pos, sc.vel)
    o.set_boundary(sc.boundary)
    out = []
    for _ in range(LARGE_REPLICA_STEPS):
        ps.Update(sc.dt)
        o.pbf_step(sc.dt, fixed_iters=LARGE_REPLICA_ITERS)
        d = ps.GetArrayVBO(abi.RX_POSITION)[:, :3].astype(np.float64) - o.get("pos")[:, :3]
        out.append(float(np.abs(d).max() / p.h))
    ps.close()
    return {"replica_particles": sc.n, "replica_boundary": int(sc.boundary.shape[0]),
            "iterations": LARGE_REPLICA_ITERS, "max_abs_position_error_over_h": out}


def large_arm(args):
    """The 16.8M-particle obstacle drop (a 256^3 block onto a box of boundary
    particles), compensated density sums, learned warm start iterating to the
    0.1 % criterion; plain form beside it; FP64 error per step on a replica."""
    import torch
    from fltk_sph_ice_gb300 import abi, build, rxPBDSPH, scenes, warmstart

    rank, world, local = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    build.build()
    L = abi.lib()
    blob, meta = warmstart.load_model(args.model)
    sc = scenes.pbf_obstacle_drop(n_side=256)
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def leg(warm: bool):
        p = abi.FsphParams.from_buffer_copy(sc.params)
        p.eta, p.error_mode, p.clamp_constraint = 1e-3, abi.ERR_ONE_SIDED, 1
        p.min_iter, p.max_iter, p.use_graph = 2, args.max_iter, 1
        p.compensated_density = 1
        p.warm_start = 1 if warm else 0
        ps = rxPBDSPH(p)
        if warm and L.fsph_set_warm_start_model(ps.handle, blob.ctypes.data_as(ctypes.c_void_p)) != abi.OK:
            raise RuntimeError("fsph_set_warm_start_model")
        ps.Set(sc.pos, sc.vel)
        ps.SetBoundary(sc.boundary)
        stats = abi.FsphStepStats()
        for _ in range(LARGE_PREROLL + max(args.warmup, 3)):
            if L.fsph_step(ps.handle, ctypes.c_float(sc.dt), sp, None) != abi.OK:
                raise RuntimeError(L.fsph_last_error(ps.handle).decode())
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        iters, errs, kern, unconv = [], [], 0, 0
        if dist:
            dist.barrier()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev[k][0].record(stream)
            L.fsph_step(ps.handle, ctypes.c_float(sc.dt), sp, None)
            ev[k][1].record(stream)
            stream.synchronize()
            L.fsph_last_stats(ps.handle, ctypes.byref(stats))
            iters.append(stats.iterations)
            errs.append(stats.density_error_one_sided)
            kern += stats.kernels
            unconv += int(stats.status == abi.NOT_CONVERGED)
        tot_s = sum(a.elapsed_time(c) for a, c in ev) / 1000.0
        value, tot_s = replica_rate(sc.n, args.steps, tot_s, dist)
        ps.close()
        return {"value": value, "ms_per_step": 1000.0 * tot_s / args.steps, "mean_iterations": float(np.mean(iters)),
                "max_error": float(np.max(errs)), "kernels": kern, "not_converged_steps": unconv,
                "status": "FSPH_NOT_CONVERGED" if unconv else "FSPH_OK"}

    with ClockSampler(local) as clk:
        plain = leg(False) if not args.no_plain else None
        warm = leg(True)
    fp64 = fp64_error_per_step(abi, rxPBDSPH, scenes) if rank == 0 and not args.no_cpu else None
    peak, peak_kind = measured_peaks()
    bytes_ps = 396.0 + 60.0 * warm["mean_iterations"]
    if rank == 0:
        cfg = {"workload": "pbf_obstacle_drop_16M", "particles": sc.n, "boundary_particles": int(sc.boundary.shape[0]),
               "block": [256, 256, 256], "dt": sc.dt, "eta_one_sided": 1e-3, "max_iter": args.max_iter,
               "compensated_density": True,
               "constraint": "unilateral (clamped C >= 0)", "method": method_of(meta),
               "mean_iterations": warm["mean_iterations"], "max_error": warm["max_error"],
               "not_converged_steps": warm["not_converged_steps"], "status": warm["status"],
               "meets_criterion": warm["not_converged_steps"] == 0,
               "preroll_steps": LARGE_PREROLL, "l2": "256 MiB flush between timed steps",
               "parallelism": f"replicas x{world}", "fp64_error_per_step": fp64}
        if plain:
            cfg["plain"] = {k: plain[k] for k in ("value", "ms_per_step", "mean_iterations", "max_error",
                                                  "not_converged_steps", "status")}
            cfg["speedup_vs_plain"] = warm["value"] / plain["value"]
        line = {
            "metric": LARGE_METRIC, "value": warm["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": warm["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
            "config": cfg,
            "roofline": {"bound": "hbm", "achieved": warm["value"] * bytes_ps / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": warm["value"] * bytes_ps / 1e9 / peak, "traffic": None, "kernel": "whole step",
                         "bytes_per_particle_step": bytes_ps, "peak_kind": peak_kind},
            "cpu_baseline": None, "e2e": None, "clocks": clk.summary(), "gpu_launches": warm["kernels"],
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--preroll", type=int, default=PREROLL)
    ap.add_argument("--model", default=None, help="warm-start network (default: the committed model)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-method leg")
    ap.add_argument("--eager", action="store_true",
                    help="host-driven iteration loop instead of the CUDA graph (same kernels; for ncu, "
                         "which cannot profile kernels inside graphs with conditional nodes)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="batched_256: skip the autotuner, default launch shape")
    ap.add_argument("--max-iter", type=int, default=2000,
                    help="pbf_obstacle_drop_16M: the constraint loop's iteration cap (a guard, default 2000: with "
                         "400 the steps after the impact stop above the tolerance and every later step inherits "
                         "their error)")
    ap.add_argument("--workload", default=WORKLOAD,
                    choices=[WORKLOAD, "batched_256", "pbf_obstacle_drop_16M", "pbf_dam_break_262k",
                             "wcsph_dam_break_32k"],
                    help="the headline 1M double dam break (default), the 256-scene batch, the 16.8M "
                         "obstacle drop with boundary particles, the 262k PBF dam break (4 iterations) or "
                         "the 32k WCSPH dam break")
    args = ap.parse_args()
    if args.model is None:
        from fltk_sph_ice_gb300 import warmstart
        args.model = warmstart.DEFAULT_MODEL
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "batched_256":
        return batched_arm(args)
    if args.workload == "pbf_obstacle_drop_16M":
        return large_arm(args)
    if args.workload in ("pbf_dam_break_262k", "wcsph_dam_break_32k"):
        return config_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
