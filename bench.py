#!/usr/bin/env python
"""Benchmark of the fluid step: PBF particle-steps/s on the 1,048,576-particle
double dam break, iterating each step until the mean one-sided density error
is <= 0.1 % (plain method; the learned warm start is selected with
--warm-start once built).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

One JSON line on rank 0.  Timing: every timed step is bracketed by CUDA events
on the stream the step is enqueued on, with a 256 MiB L2 flush between steps
(outside the events); max over ranks; W >= 3 untimed warm-up steps after a
100-step pre-roll that brings the dam break into its collapsing phase.
Multi-GPU runs are independent replicas (the path does not shard; weak scaling).

Legs of the line:
  value / ms_per_step  device-resident steps (graph launch per step)
  e2e                  the same steps through the public API with the particle
                       state crossing host<->device every step (pinned buffers)
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
# constraint iterations per step of the reference CPU arm (eta = 0 makes its
# loop run exactly this many); the plain GPU method averages about this many
# iterations per step on the timed window of this workload
REF_ITERS = 8
# algorithmic (compulsory) bytes per particle of one launch
BYTES_LAMBDA = 24.0       # R x* 16, W lambda 4, W rho 4
BYTES_CORRECTION = 36.0   # R x* 16, R lambda 4, W x* 16


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


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


def reference_arm(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    block = (20, 20, 40)
    sc = make_scene(block)
    n = sc.n
    for _ in range(max(args.warmup, 0)):
        cpu_sample(sc.pos, sc.vel, sc.params, REF_ITERS)
    times = []
    kind = "reference"
    for _ in range(args.steps):
        t, kind = cpu_sample(sc.pos, sc.vel, sc.params, REF_ITERS)
        times.append(t)
    tot = sum(times)
    value = n * len(times) / tot
    sample = (f"one PBF step of the {n}-particle double dam break (blocks {block[0]}x{block[1]}x{block[2]}, "
              f"initial state) per timed step, {REF_ITERS} fixed constraint iterations, 1 host thread")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "sample_particles": n, "iterations": REF_ITERS},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def gpu_arm(args):
    import torch
    from fltk_sph_ice_gb300 import abi, build, rxPBDSPH

    rank, world, local = rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    build.build()
    L = abi.lib()

    sc = make_scene(warm_start=1 if args.warm_start else 0)
    if args.eager:
        sc.params.use_graph = 0
    n = sc.n
    dt = sc.dt
    ps = rxPBDSPH(sc.params)
    ps.Set(sc.pos, sc.vel)
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    stats = abi.FsphStepStats()

    def step(with_stats=False):
        st = L.fsph_step(ps.handle, ctypes.c_float(dt), sp, ctypes.byref(stats) if with_stats else None)
        if st != abi.OK:
            raise abi.FsphError(st, L.fsph_last_error(ps.handle).decode())

    for _ in range(args.preroll):
        step()
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    iters, errs = [], []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
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
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tot_ms = sum(step_ms)
    if dist:
        t = torch.tensor([tot_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = n * args.steps * world / (tot_ms / 1000.0)
    mean_iters = float(np.mean(iters))
    clocks = clk.summary()

    # ---- roofline of the dominant kernel (event-timed launches on the context stream)
    t_lam = ctypes.c_float(0)
    t_cor = ctypes.c_float(0)
    t_grid = ctypes.c_float(0)
    state_pos = ps.GetArrayVBO(abi.RX_POSITION)
    state_vel = ps.GetArrayVBO(abi.RX_VELOCITY)
    L.fsph_time_pass(ps.handle, abi.PASS_LAMBDA, 20, ctypes.byref(t_lam))
    L.fsph_time_pass(ps.handle, abi.PASS_CORRECTION, 20, ctypes.byref(t_cor))
    L.fsph_time_pass(ps.handle, abi.PASS_GRID, 10, ctypes.byref(t_grid))
    lam_share = mean_iters * t_lam.value
    cor_share = mean_iters * t_cor.value
    if cor_share >= lam_share:
        kname, kms, kbytes = "k_correction", t_cor.value, BYTES_CORRECTION * n
    else:
        kname, kms, kbytes = "k_lambda", t_lam.value, BYTES_LAMBDA * n
    peak, peak_kind = measured_peaks()
    achieved = kbytes / (kms / 1000.0) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.isfile(tp):
        with open(tp) as f:
            tr = json.load(f)
        if kname in tr:
            traffic = tr[kname].get("bytes_per_launch_1M")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": kname, "launch_ms": kms, "peak_kind": peak_kind,
                "lambda_ms": t_lam.value, "correction_ms": t_cor.value, "grid_build_ms": t_grid.value}

    # ---- e2e: the public API with host buffers every step
    e2e = None
    if not args.no_e2e:
        pin_pos = torch.from_numpy(state_pos).pin_memory().numpy()
        pin_vel = torch.from_numpy(state_vel).pin_memory().numpy()
        out_pos = torch.empty((n, 4), dtype=torch.float32).pin_memory().numpy()
        out_vel = torch.empty((n, 4), dtype=torch.float32).pin_memory().numpy()
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731

        def e2e_step():
            st = L.fsph_set_particles(ps.handle, vp(pin_pos), vp(pin_vel), n, abi.HOST)
            st |= L.fsph_step(ps.handle, ctypes.c_float(dt), None, None)
            st |= L.fsph_get_array(ps.handle, abi.RX_POSITION, vp(out_pos), abi.HOST, None)
            st |= L.fsph_get_array(ps.handle, abi.RX_VELOCITY, vp(out_vel), abi.HOST, None)
            if st != abi.OK:
                raise abi.FsphError(st, L.fsph_last_error(ps.handle).decode())
            np.copyto(pin_pos, out_pos)
            np.copyto(pin_vel, out_vel)

        for _ in range(3):
            e2e_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e2e_s = time.perf_counter() - t0
        if dist:
            t = torch.tensor([e2e_s], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        e2e = {"value": n * args.steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * 16 * n,
               "d2h_bytes_per_step": 2 * 16 * n}

    # ---- CPU baseline (rank 0, single GPU only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        block = (20, 20, 40)
        sm = make_scene(block)
        ps2 = rxPBDSPH(sm.params)
        ps2.Set(sm.pos, sm.vel)
        for _ in range(args.preroll):
            ps2.Update(sm.dt, stats=False)
        xs, vs = ps2.GetArrayVBO(abi.RX_POSITION), ps2.GetArrayVBO(abi.RX_VELOCITY)
        ps2.close()
        ci = max(1, int(round(mean_iters)))
        secs, kind = cpu_sample(xs, vs, sm.params, ci)
        cpu = {"value": sm.n / secs, "unit": UNIT, "cores": 1, "kind": kind,
               "sample": (f"one PBF step of the {sm.n}-particle double dam break (blocks {block[0]}x{block[1]}x{block[2]}) "
                          f"after the same {args.preroll}-step pre-roll, {ci} fixed constraint iterations "
                          f"(the GPU mean), 1 host thread")}

    launches_per_iter = 2
    launches_fixed = 8 + (2 if (sc.params.xsph_c or sc.params.vort_eps) else 0)
    gpu_launches = int(args.steps * (launches_fixed + launches_per_iter * mean_iters))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded jittered lattices)",
            "config": {"workload": WORKLOAD, "particles": n, "block": list(BLOCK), "dt": dt,
                       "eta_one_sided": 1e-3, "constraint": "unilateral (clamped C >= 0)",
                       "mean_iterations": mean_iters, "max_error": float(np.max(errs)),
                       "warm_start": bool(args.warm_start), "preroll_steps": args.preroll,
                       "l2": "256 MiB flush between timed steps", "parallelism": f"replicas x{world}"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": gpu_launches,
        }
        print(json.dumps(line), flush=True)
    ps.close()
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
    ap.add_argument("--warm-start", action="store_true")
    ap.add_argument("--eager", action="store_true",
                    help="host-driven iteration loop instead of the CUDA graph (same kernels; for ncu, "
                         "which cannot profile kernels inside graphs with conditional nodes)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
