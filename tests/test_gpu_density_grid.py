"""The density field on a lattice for surface meshing (fsph_density_grid;
CalImplicitField / GetImplicit, rx_sph_pbd.cpp:2024-2108) on the GPU against
the reference's own CalImplicitField (oracle/_ref) and the oracle."""
import numpy as np
import pytest

import oracle
from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes

pytestmark = pytest.mark.gpu


def test_density_grid_matches_reference_and_oracle(gpu):
    """CalImplicitField on the GPU (fsph_density_grid) against the
    reference's own CalImplicitField and the oracle, on a collapsing dam;
    GetImplicit at a node agrees with the lattice."""
    from test_density_grid_oracle import lattice
    sc = scenes.pbf_double_dam_break(block=(16, 16, 32))
    p = sc.params
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    for _ in range(30):
        ps.Update(sc.dt)
    x = ps.GetArrayVBO(abi.RX_POSITION)
    nn, lo, d = lattice(p, (96, 30, 50))
    got = ps.CalImplicitField(nn, lo, d)
    ref = oracle.RefSolver(p, sc.n, "pbf").density_grid(x, nn, lo, d)
    o = oracle.Oracle(p, sc.n, threads=4)
    o.set(x)
    orc = o.density_grid(nn, lo, d)
    assert (ref > 0).sum() > 10000
    assert np.abs(got - ref).max() <= 1e-6 * ref.max(), np.abs(got - ref).max() / ref.max()
    assert np.abs(got - orc).max() <= 1e-6 * ref.max()
    k, j, i = 15, 5, 40
    pt = [lo[0] + i * d[0], lo[1] + j * d[1], lo[2] + k * d[2]]
    assert abs(ps.GetImplicit(*pt) - got[k, j, i]) <= 1e-6 * ref.max()
