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
from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes

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
