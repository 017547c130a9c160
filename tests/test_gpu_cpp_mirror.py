"""The C++ drop-in classes (include/fsph_particle_system.hpp) driven by a
reference-style C++ program, against the same steps through the Python
mirror and the CPU oracle; the particle file is the reference's binary
format (rx_ps.cpp:581-644)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT, assert_rel
from fltk_sph_ice_gb300 import abi, rxPBDSPH, rxSPH, scenes

pytestmark = pytest.mark.gpu


def write_particles(fn, pos, vel):
    with open(fn, "wb") as f:
        np.array([pos.shape[0]], np.uint32).tofile(f)
        np.ascontiguousarray(pos[:, :3], np.float32).tofile(f)
        np.ascontiguousarray(vel[:, :3], np.float32).tofile(f)


def read_particles(fn):
    with open(fn, "rb") as f:
        n = int(np.fromfile(f, np.uint32, 1)[0])
        p = np.fromfile(f, np.float32, 3 * n).reshape(n, 3)
        v = np.fromfile(f, np.float32, 3 * n).reshape(n, 3)
    return p, v


def test_cpp_driver_matches_python_and_oracle(gpu, tmp_path):
    exe = tmp_path / "pbf_driver"
    lib_dir = os.path.dirname(abi.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "pbf_driver.cpp"), "-L", lib_dir, "-lfsph",
                    f"-Wl,-rpath,{lib_dir}", "-L/usr/local/cuda/lib64", "-lcudart", "-o", str(exe)], check=True)
    sc = scenes.pbf_double_dam_break(block=(10, 10, 20))
    p = sc.params
    p.eta, p.max_iter = 0.0, 4
    vel = np.zeros_like(sc.pos)
    vel[:, 1] = -0.3
    (tmp_path / "params.bin").write_bytes(bytes(p))
    write_particles(tmp_path / "in.dat", sc.pos, vel)
    r = subprocess.run([str(exe), str(tmp_path / "params.bin"), str(tmp_path / "in.dat"), str(tmp_path / "out.dat"),
                        "3", repr(sc.dt)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("iterations 4") == 3
    cpos, cvel = read_particles(tmp_path / "out.dat")

    ps = rxPBDSPH(p)
    ps.Set(sc.pos, vel)
    for _ in range(3):
        ps.Update(sc.dt)
    np.testing.assert_array_equal(cpos, ps.GetArrayVBO(abi.RX_POSITION)[:, :3])
    np.testing.assert_array_equal(cvel, ps.GetArrayVBO(abi.RX_VELOCITY)[:, :3])
    off, idx = ps.GetNeights()
    assert f"neighbours {len(idx)}" in r.stdout

    o = oracle.Oracle(p, sc.n, threads=4)
    o.set(sc.pos, vel)
    for _ in range(3):
        o.pbf_step(sc.dt)
    assert_rel(cpos, o.get("pos")[:, :3], 1e-5, "C++ driver positions vs oracle")


def test_reference_style_caller_runs(gpu, tmp_path):
    """tests/cpp/ref_style_caller.cpp: the InitSPH / SetLiquidBox / StepPS
    sequence of the reference's application through a base-class pointer,
    then the neighbour lists, UpdateWithoutPosAndVel and the particle file."""
    exe = tmp_path / "ref_style_caller"
    lib_dir = os.path.dirname(abi.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "ref_style_caller.cpp"), "-L", lib_dir, "-lfsph",
                    f"-Wl,-rpath,{lib_dir}", "-L/usr/local/cuda/lib64", "-lcudart", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), str(tmp_path / "out.dat"), "20"], capture_output=True, text=True)
    print(r.stderr)
    assert r.returncode == 0, r.stderr
    f = r.stdout.split()
    vals = {f[k]: f[k + 1] for k in range(0, 12, 2)}
    n = int(vals["particles"])
    assert n == 13 ** 3                      # AddBox: (2 sx + 1)^3 with sx = (int)(0.2 / 2r) - 1 = 6
    assert int(vals["max"]) == 20000
    assert int(vals["neighbours"]) > 10 * n  # ~20 per interior particle at the lattice spacing 2r, fewer at the surface
    assert float(vals["dist_check"]) < 2.5e-7  # Dist = fl32(sqrt(Dist2)): Dist^2 within ~1 ulp of Dist2
    assert int(vals["unmoved"]) == 1          # UpdateWithoutPosAndVel leaves the particles
    assert f[10] == "density" and f[13] == "dim" and f[17] == "resume"
    rho_min, rho_max = float(f[11]), float(f[12])
    assert int(f[18]) == 1  # SaveCheckpoint / LoadCheckpoint: five more steps bit-identical
    assert 0 < rho_min < rho_max < 2000.0
    pos, vel = read_particles(tmp_path / "out.dat")
    assert pos.shape == (n, 3) and np.isfinite(pos).all() and np.isfinite(vel).all()


def test_update_without_pos_and_vel(gpu):
    """UpdateWithoutPosAndVel: the fields of a step (WCSPH density, pressure,
    acceleration; PBF pre-pass density and external + viscous acceleration)
    against the oracle, particles unchanged."""
    sw = scenes.wcsph_dam_break(n_side=12)
    ws = rxSPH(sw.params)
    ws.Set(sw.pos, sw.vel)
    ws.UpdateWithoutPosAndVel(sw.dt)
    o = oracle.Oracle(sw.params, sw.n)
    d, pr, a = o.sph_forces(sw.pos, sw.vel)
    assert_rel(ws.GetArrayVBO(abi.RX_DENSITY), d, 1e-5, "WCSPH density")
    assert_rel(ws.GetArrayVBO(abi.RX_PRESSURE), pr, 1e-5, "WCSPH pressure")
    assert_rel(ws.GetArrayVBO(abi.RX_FORCE), a, 1e-5, "WCSPH acceleration")
    np.testing.assert_array_equal(ws.GetArrayVBO(abi.RX_POSITION), sw.pos)
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    p = sc.params
    p.viscosity = 0.05
    vel = np.zeros_like(sc.pos)
    vel[:, 0] = 0.3
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, vel)
    ps.UpdateWithoutPosAndVel(sc.dt)
    o2 = oracle.Oracle(p, sc.n)
    o2.set(sc.pos, vel)
    d2, f2, _, _ = o2.pbf_predict(sc.dt)
    assert_rel(ps.GetArrayVBO(abi.RX_DENSITY), d2, 1e-5, "PBF density")
    assert_rel(ps.GetArrayVBO(abi.RX_FORCE)[:, :3], f2[:, :3], 1e-5, "PBF external + viscous acceleration")
    np.testing.assert_array_equal(ps.GetArrayVBO(abi.RX_POSITION), sc.pos)
