"""The oracle's density field on a lattice (for meshing) against the
reference's own rxPBDSPH::CalImplicitField -> CalColorField
(rx_sph_pbd.cpp:2024-2108), compiled here from its sources (oracle/_ref):
CPU only.  Bar: 1e-6 relative to the largest node value (the two visit the
neighbours in different orders; the sums are float)."""
import numpy as np
import pytest

import oracle
from fltk_sph_ice_gb300 import scenes


def lattice(p, nn=(40, 14, 22), margin=0.03):
    lo = [p.box_min[a] - margin for a in range(3)]
    d = [(p.box_max[a] - p.box_min[a] + 2 * margin) / (nn[a] - 1) for a in range(3)]
    return list(nn), lo, d


def test_density_grid_matches_reference():
    if oracle.ref_lib() is None:
        pytest.skip("the reference-code library is not built on this host")
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    p = sc.params
    o = oracle.Oracle(p, sc.n, threads=4)
    o.set(sc.pos, sc.vel)
    for _ in range(10):
        o.pbf_step(sc.dt)
    x = o.get("pos")
    nn, lo, d = lattice(p)
    got = o.density_grid(nn, lo, d)
    want = oracle.RefSolver(p, sc.n, "pbf").density_grid(x, nn, lo, d)
    assert (want > 0).sum() > 500 and (want == 0).sum() > 500
    assert np.abs(got - want).max() <= 1e-6 * want.max()
    # the nodes outside the simulation range (the box grown by 1 %) read 0
    assert (got[:, :, 0] == 0).all() and (got[:, :, -1] == 0).all()
