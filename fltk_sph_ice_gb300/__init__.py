"""GB300-native fluid step of fltk_sph_ice.

The hashed-grid neighbour search, the WCSPH density / pressure / viscosity
pass and the PBF density-constraint iterations of the reference simulator
(rx_sph_cpu.cpp, rx_sph_pbd.cpp, rx_sph_kernel.cu, rx_pbdsph_kernel.cu), as
sm_103a CUDA kernels behind a C ABI (include/fsph.h, libfsph.so).

    from fltk_sph_ice_gb300 import rxPBDSPH, scenes
    sc = scenes.pbf_dam_break(32)
    ps = rxPBDSPH(sc.params); ps.Set(sc.pos); ps.Update(sc.dt)
"""
from . import abi, scenes
from .abi import FsphError
from .batch import PBFBatch
from .particles import rxParticleSystemBase, rxPBDSPH, rxSPH

__all__ = ["abi", "scenes", "FsphError", "PBFBatch", "rxParticleSystemBase", "rxPBDSPH", "rxSPH"]
