"""The C++ drop-in header compiles on its own (g++: no GPU needed), with the
calls a reference-style driver makes: the older fsph_params-based calls, a
caller written the way the reference's application drives its particle
system (tests/cpp/ref_style_caller.cpp, compiled and linked against
libfsph.so), and a caller that brings its own vector type."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = r'''
#include "fsph_particle_system.hpp"
#include <vector>
using namespace fsph_gb300;
int drive(const fsph_params &p) {
    rxPBDSPH ps(p);
    std::vector<float> pos(3 * 8, 0.0f), vel(3 * 8, 0.0f), blob(FSPH_MLP_BLOB_SIZE, 0.0f), bnd(4 * 2, 0.0f);
    ps.Set(pos, vel);
    ps.SetBoundary(bnd);
    ps.SetWarmStartModel(blob);
    ps.Update(0.0016f);
    float *x = ps.GetArrayVBO(rxParticleSystemBase::RX_POSITION);
    ps.SetArrayVBO(rxParticleSystemBase::RX_POSITION, x, 0, ps.GetNumParticles());
    return ps.GetNumBoundaryParticles() + (int)ps.GetBoundary(FSPH_BOUNDARY_VOLUME).size();
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_cpp_dropin_header_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text(SRC)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


OWN_VEC = r'''
#include "fsph_particle_system.hpp"
#include <vector>
/* a caller-side vector type with operator[], as the reference's Vec3 */
struct MyVec { double v[3]; double operator[](int i) const { return v[i]; } };
int drive() {
    fsph_gb300::rxParticleSystemBase *ps = new fsph_gb300::rxSPH(false);
    fsph_gb300::rxSPHEnviroment env;
    ((fsph_gb300::rxSPH *)ps)->Initialize(env);
    std::vector<MyVec> p(4, MyVec{{0.0, 0.1, 0.2}}), v(4, MyVec{{0.0, 0.0, 0.0}});
    ((fsph_gb300::rxSPH *)ps)->Set(p, v);
    MyVec c{{0.0, 0.0, 0.0}}, e{{0.1, 0.1, 0.1}};
    ps->AddBox(-1, c, e, MyVec{{0.0, 0.0, 0.0}}, 0.02f);
    float pos[4] = {0, 0, 0, 0}, vel[4] = {0, 0, 0, 0};
    ps->AddSphere(0, pos, vel, 2, 0.02f);
    ps->Reset(fsph_gb300::rxParticleSystemBase::RX_CONFIG_GRID);
    ps->SetParticlesToCell(pos, 1, 0.05f);
    int n = ps->GetNumParticles();
    delete ps;
    fsph_gb300::rxPBDSPH pbf(false);
    pbf.Initialize(env);
    pbf.GetArtificialPressure() = false;  /* rx_sph.h:1199 */
    return n + pbf.GetNumParticles();
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_reference_style_caller_compiles_and_links(tmp_path):
    from fltk_sph_ice_gb300 import build
    lib = build.build()
    exe = tmp_path / "ref_style_caller"
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-Wextra", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "ref_style_caller.cpp"), "-L", os.path.dirname(lib),
                        "-lfsph", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_caller_vector_type_accepted(tmp_path):
    src = tmp_path / "own_vec.cpp"
    src.write_text(OWN_VEC)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
