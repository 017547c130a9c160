"""The C++ drop-in header compiles on its own (g++, syntax only: no GPU and
no library needed), with the calls a reference-style driver makes."""
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
