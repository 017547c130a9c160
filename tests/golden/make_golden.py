"""Generate tests/golden/*.npz from the reference's OWN CPU fluid code.

Runs the functions compiled into oracle/_ref/libfsph_ref.so (the
reference's rx_nnsearch.h / rx_sph_pbd.cpp / rx_sph_cpu.cpp /
rx_sph_solid.cpp / rx_kernel.h, see oracle/ref_harness/extract.py) on small
seeded states and stores inputs and outputs.  Needs the reference tree (or
an already extracted oracle/_ref/src) -- the fixtures themselves are
committed so that the tests need neither.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from fltk_sph_ice_gb300 import scenes  # noqa: E402


def compressed(pos: np.ndarray, factor: float) -> np.ndarray:
    """Squeeze a block toward its centroid (creates a non-trivial constraint state)."""
    out = pos.copy()
    c = out[:, :3].mean(axis=0)
    out[:, :3] = (c + (out[:, :3] - c) * factor).astype(np.float32)
    return out


def pbf_case():
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    p = sc.params
    p.eta = 0.0          # the tolerance loop then runs exactly max_iter iterations
    p.min_iter = 2
    p.max_iter = 4
    p.error_mode = 1     # the CPU path's two-sided error
    p.xsph_c = 0.0
    p.vort_eps = 0.0
    n = sc.n
    x = compressed(sc.pos, 0.97)
    ref = oracle.RefSolver(p, n, "pbf")
    off, idx, d2 = ref.neighbors(x)
    dens, lam = ref.lambda_pass(x, sc.dt)
    dp = ref.correction_pass(x, lam, sc.dt)
    ref2 = oracle.RefSolver(p, n, "pbf")
    vel = np.zeros_like(x)
    vel[:, 1] = -0.5
    ref2.set(x, vel)
    pd, pf, ppos, pvel = ref2.pbf_predict(sc.dt)
    ref3 = oracle.RefSolver(p, n, "pbf")
    ref3.set(x, vel)
    its, etas, traj = [], [], []
    for _ in range(3):
        it, eta = ref3.update(sc.dt)
        its.append(it)
        etas.append(eta)
        traj.append(ref3.get("pos"))
    return dict(
        pos=x, vel=vel, dt=np.float32(sc.dt), params=np.frombuffer(bytes(p), dtype=np.uint8),
        nb_off=off, nb_idx=idx, nb_dist2=d2, dens=dens, lam=lam, dp=dp,
        pre_dens=pd, pre_frc=pf, pre_ppos=ppos, pre_pvel=pvel,
        step_iters=np.array(its, np.int32), step_eta=np.array(etas, np.float64),
        step_pos=np.stack(traj), step_vel_last=ref3.get("vel"),
    )


def sph_case():
    sc = scenes.wcsph_dam_break(n_side=10)
    p = sc.params
    n = sc.n
    x = compressed(sc.pos, 0.98)
    vel = np.zeros_like(x)
    vel[:, 0] = 0.3
    ref = oracle.RefSolver(p, n, "sph")
    ref.set(x, vel)
    dens, pres, frc = ref.sph_forces()
    ref2 = oracle.RefSolver(p, n, "sph")
    ref2.set(x, vel)
    traj = []
    for _ in range(5):
        ref2.update(sc.dt)
        traj.append(ref2.get("pos"))
    return dict(
        pos=x, vel=vel, dt=np.float32(sc.dt), params=np.frombuffer(bytes(p), dtype=np.uint8),
        dens=dens, pres=pres, frc=frc, step_pos=np.stack(traj), step_vel_last=ref2.get("vel"),
    )


def kernel_case():
    L = oracle.ref_lib()
    h = 0.0457
    r = np.linspace(0.0, 1.1 * h, 97)
    w = np.array([L.fsph_ref_kernel(0, float(x), h) for x in r])
    g = np.array([L.fsph_ref_kernel(1, float(x), h) for x in r])
    lap = np.array([L.fsph_ref_kernel(2, float(x), h) for x in r])
    # box wall: face, edge and corner violations plus an interior point
    cen = np.array([0.5, 0.3, 0.2])
    ext = np.array([0.5, 0.3, 0.2])
    pts = np.array([[0.5, 0.3, 0.2], [-0.01, 0.3, 0.2], [1.02, 0.3, 0.2], [0.5, -0.05, 0.2],
                    [-0.02, -0.03, 0.2], [1.01, 0.61, 0.41], [-0.1, 0.7, -0.3], [0.001, 0.3, 0.2]])
    rad = 0.015625  # exactly representable in float, as the solvers store the radius
    wall = np.zeros_like(pts)
    hit = np.zeros(len(pts), np.int32)
    import ctypes
    for i, q in enumerate(pts):
        o = np.zeros(3)
        hit[i] = L.fsph_ref_wall(cen.ctypes.data_as(ctypes.c_void_p), ext.ctypes.data_as(ctypes.c_void_p), rad,
                                 q.ctypes.data_as(ctypes.c_void_p), o.ctypes.data_as(ctypes.c_void_p))
        wall[i] = o
    return dict(h=np.float64(h), r=r, poly6=w, spiky_g=g, visc_lap=lap, wall_cen=cen, wall_ext=ext,
                wall_r=np.float64(rad), wall_pts=pts, wall_out=wall, wall_hit=hit)


def main():
    if oracle.ref_lib() is None:
        raise SystemExit("reference CPU code unavailable: cannot regenerate golden vectors")
    for name, fn in (("pbf_small", pbf_case), ("sph_small", sph_case), ("kernels", kernel_case)):
        d = fn()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: getattr(v, "shape", ()) for k, v in d.items()})


if __name__ == "__main__":
    main()
