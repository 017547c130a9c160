"""The C-ABI library without a GPU: it builds, loads, exports every symbol
include/fsph.h declares, its structs match the ctypes mirror, and its
host-only entry points (status strings, parameter derivation) behave.
No compute call is made here."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT, cuda_device_count
from fltk_sph_ice_gb300 import abi

HEADER = os.path.join(ROOT, "include", "fsph.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w ]+?\**\s*\b(fsph_\w+)\s*\(", src, flags=re.M)))


def test_exports_every_declared_symbol(fsph):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fsph_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert set(names) == set(abi.EXPORTS)


def test_debug_bounds_library_exports_the_same_symbols(fsph):
    """the FSPH_DEBUG_BOUNDS build is the same library with checks added"""
    from fltk_sph_ice_gb300 import build
    path = build.build(debug_bounds=True)
    assert path != abi.LIB_PATH and os.path.isfile(path)
    syms = [set(re.findall(r" T (fsph_\w+)", subprocess.run(["nm", "-D", "--defined-only", p], capture_output=True,
                                                           text=True).stdout)) for p in (abi.LIB_PATH, path)]
    assert syms[0] == syms[1] and set(declared_functions()) <= syms[1]


def test_struct_layout_matches_header(tmp_path):
    c = tmp_path / "sz.c"
    c.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "fsph.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(fsph_params), sizeof(fsph_env),"
        " sizeof(fsph_step_stats), offsetof(fsph_params, box_min), offsetof(fsph_params, cell_skin),"
        " offsetof(fsph_env, dens));return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(abi.FsphParams), ctypes.sizeof(abi.FsphEnv), ctypes.sizeof(abi.FsphStepStats),
            abi.FsphParams.box_min.offset, abi.FsphParams.cell_skin.offset, abi.FsphEnv.dens.offset]
    assert got == want


def test_status_strings(fsph):
    for code, name in abi.STATUS_NAMES.items():
        assert fsph.fsph_status_string(code).decode() == name
    assert fsph.fsph_abi_version() == 1


def test_params_from_env_matches_reference_initialize(fsph):
    """fsph_params_from_env derives h, r and rho0 as rxPBDSPH::Initialize does."""
    e = abi.FsphEnv()
    e.solver = abi.SOLVER_PBF
    e.max_particles = 1000
    for a, (c, x) in enumerate(zip((0.0, 0.0, 0.0), (0.5, 0.3, 0.2))):
        e.boundary_cen[a] = c
        e.boundary_ext[a] = x
    e.dens, e.mass, e.kernel_particles = 998.29, 0.02, 20.0
    e.viscosity, e.gas_k, e.epsilon, e.eta = 1e-3, 3.0, 0.001, 0.05
    e.min_iter, e.max_iter, e.use_ap, e.ap_k, e.ap_n, e.ap_q, e.gravity_y = 2, 10, 1, 0.1, 4.0, 0.2, -9.81
    p = abi.FsphParams()
    assert fsph.fsph_params_from_env(ctypes.byref(e), ctypes.byref(p)) == abi.OK
    # known answer (also printed by the reference's Initialize): h = 0.04573, rho0 = 961.2326
    assert abs(p.h - 0.0457339) < 1e-6
    assert abs(p.rest_dens - 961.2325) < 1e-3
    assert p.box_min[0] == -0.5 and p.box_max[1] == 0.3
    L = oracle.ref_lib()
    if L is None:
        pytest.skip("reference CPU code unavailable for the live comparison")
    env = oracle.RefEnv()
    env.max_particles = 1000
    for a in range(3):
        env.boundary_cen[a], env.boundary_ext[a] = e.boundary_cen[a], e.boundary_ext[a]
    env.dens, env.mass, env.kernel_particles = e.dens, e.mass, e.kernel_particles
    env.max_iter, env.min_iter, env.use_ap, env.ap_q = 10, 2, 1, 0.2
    h = L.fsph_ref_pbf_create(ctypes.byref(env))
    out = np.zeros(13)
    L.fsph_ref_pbf_scalars(h, out.ctypes.data_as(ctypes.c_void_p))
    L.fsph_ref_pbf_destroy(h)
    assert np.float32(out[0]) == np.float32(p.h)
    assert np.float32(out[1]) == np.float32(p.particle_radius)
    assert abs(out[2] - p.rest_dens) <= 1e-6 * out[2]


def test_create_without_device_reports_no_device(fsph):
    if cuda_device_count() > 0:
        pytest.skip("a CUDA device is present")
    p = abi.FsphParams()
    fsph.fsph_params_default(ctypes.byref(p))
    p.max_particles = 10
    ctx = ctypes.c_void_p()
    assert fsph.fsph_create(ctypes.byref(p), ctypes.byref(ctx)) == abi.NO_DEVICE
    assert not ctx.value


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        abi.lib(str(tmp_path / "libfsph.so"))
