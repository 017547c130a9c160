"""Dynamic particle count on the GPU: inlet lines (AddLine / addParticles,
rx_ps.cpp:432-520) and deletion regions (checkDeletePB,
rx_pbdsph_kernel.cu:1171-1187), and deletion through the attribute."""
import numpy as np
import pytest

from conftest import assert_rel
from fltk_sph_ice_gb300 import FsphError, abi, rxPBDSPH, rxSPH, scenes

pytestmark = pytest.mark.gpu


def base(n_max, solver="pbf"):
    h = scenes.H_DEFAULT
    p = scenes.pbf_params(h, [0, 0, 0], [0.6, 0.5, 0.3], n_max)
    p.eta, p.min_iter, p.max_iter = 1e-3, 2, 20
    if solver == "sph":
        p.solver = abi.SOLVER_WCSPH
        p.mass, p.viscosity = 0.02, 3.5 / scenes.REST_DENS
    return p


def inlet_numpy(pos1, pos2, up, accum, spacing_rows, r):
    """The placement of addParticles without the jitter."""
    pos1, pos2, up = (np.asarray(v, np.float64) for v in (pos1, pos2, up))
    rel = pos2 - pos1
    l = np.linalg.norm(rel)
    n = int(l / r)
    sp = l / n
    out = []
    p1 = pos1.copy()
    for _ in range(accum):
        for i in range(n):
            out.append(p1 + rel / l * (i + 0.5) * sp)
        p1 = p1 + up * spacing_rows * sp
    return np.array(out), sp


@pytest.mark.parametrize("solver", ["pbf", "sph"])
def test_inlet_lines_add_particles(gpu, solver):
    p = base(4000, solver)
    cls = rxPBDSPH if solver == "pbf" else rxSPH
    ps = cls(p)
    r = float(np.float32(p.particle_radius))
    line = dict(pos1=(0.1, 0.3, 0.1), pos2=(0.1, 0.3, 0.2), vel=(0.5, 0.0, 0.0), up=(0.0, 1.0, 0.0), accum=3, span=2,
                spacing=2.0)
    assert ps.AddLine(**line) == 1
    want, sp = inlet_numpy(line["pos1"], line["pos2"], line["up"], line["accum"], line["spacing"], r)
    assert ps.EmitInlets(1) == 0            # 1 % span != 0
    assert ps.EmitInlets(2) == len(want)
    x = ps.GetArrayVBO(abi.RX_POSITION)[:, :3]
    assert x.shape[0] == len(want) == ps.GetNumActiveParticles()
    assert np.abs(x - want).max() <= 0.0101 * sp     # the jitter bound, 0.01 of the spacing
    assert (ps.GetArrayVBO(abi.RX_ATTRIBUTE) == 0).all()
    np.testing.assert_allclose(ps.GetArrayVBO(abi.RX_VELOCITY)[:, :3], np.tile([0.5, 0.0, 0.0], (len(want), 1)))
    dt = 0.0016 if solver == "pbf" else 0.001
    for step in range(3, 40):
        ps.Update(dt, step)  # the line emits on the even steps, 4 to 38
    n = ps.GetNumParticles()
    assert n == len(want) * (1 + 18) and ps.GetNumActiveParticles() == n
    assert np.isfinite(ps.GetArrayVBO(abi.RX_POSITION)).all()
    # past max_particles the emission wraps and overwrites from index 0
    while ps.GetNumParticles() + len(want) <= 4000:
        ps.EmitInlets(0)
    before = ps.GetArrayVBO(abi.RX_POSITION)
    ps.EmitInlets(0)
    assert ps.GetNumParticles() == 4000
    after = ps.GetArrayVBO(abi.RX_POSITION)
    k = ps.GetNumParticles() - (before.shape[0])
    assert not np.array_equal(after[:len(want) - k], before[:len(want) - k])  # the oldest were replaced


def test_deletion_regions(gpu):
    sc = scenes.pbf_double_dam_break(block=(10, 10, 20))
    p = sc.params
    p.max_iter = 30
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    L = [p.box_max[a] for a in range(3)]
    # a region at the floor in the middle of the tank: the fronts run into it
    lo, hi = (0.4 * L[0], -1.0, -1.0), (0.6 * L[0], 0.3 * L[1], 2.0)
    ps.AddDeleteRegion(lo, hi)
    deleted_at = None
    for k in range(150):
        ps.Update(sc.dt)
        if ps.GetNumActiveParticles() < sc.n and deleted_at is None:
            deleted_at = k
    assert deleted_at is not None and ps.GetNumParticles() == sc.n
    attr = ps.GetArrayVBO(abi.RX_ATTRIBUTE)
    x = ps.GetArrayVBO(abi.RX_POSITION)
    gone = attr == -1
    assert gone.sum() == sc.n - ps.GetNumActiveParticles() > 0
    np.testing.assert_array_equal(x[gone, :3], np.tile([0.0, 0.0, 1e6], (gone.sum(), 1)))
    assert (ps.GetArrayVBO(abi.RX_VELOCITY)[gone] == 0).all()
    live = x[~gone, :3]
    inside = ((live > np.array(lo)) & (live < np.array(hi))).all(1)
    assert not inside.any()
    # the active particles step as the same particles would on their own
    xa, va = live.copy(), ps.GetArrayVBO(abi.RX_VELOCITY)[~gone]
    solo = rxPBDSPH(p)
    solo.Set(xa, va)
    ps.Update(sc.dt)
    solo.Update(sc.dt)
    x2 = ps.GetArrayVBO(abi.RX_POSITION)[~gone, :3]
    attr2 = ps.GetArrayVBO(abi.RX_ATTRIBUTE)
    still = attr2[~gone] != -1  # the ones this step did not delete
    assert_rel(x2[still], solo.GetArrayVBO(abi.RX_POSITION)[still, :3], 1e-5, "active particles vs alone")


def test_attribute_deletes_and_revives(gpu):
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    ps = rxPBDSPH(sc.params)
    ps.Set(sc.pos, sc.vel)
    ps.Update(sc.dt)
    a = ps.GetArrayVBO(abi.RX_ATTRIBUTE)
    a[:100] = -1
    ps.SetArrayVBO(abi.RX_ATTRIBUTE, a)
    assert ps.GetNumActiveParticles() == sc.n - 100
    x0 = ps.GetArrayVBO(abi.RX_POSITION)
    ps.Update(sc.dt)
    x1 = ps.GetArrayVBO(abi.RX_POSITION)
    np.testing.assert_array_equal(x1[:100], x0[:100])  # deleted: no longer moved
    assert not np.array_equal(x1[100:], x0[100:])
    a[:100] = 0
    ps.SetArrayVBO(abi.RX_ATTRIBUTE, a)
    assert ps.GetNumActiveParticles() == sc.n
    with pytest.raises(FsphError):
        ps.AddLine((0, 0, 0), (1, 0, 0), (0, 0, 0), (0, 1, 0), 0, 1, 1.0)  # accum >= 1
