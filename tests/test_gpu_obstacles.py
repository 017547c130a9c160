"""Analytic box and sphere obstacles on the GPU (fsph_set_box_obstacle /
fsph_set_sphere_obstacle; SetBoxObstacle / SetSphereObstacle, rx_ps.h:266-272)
against the CPU oracle, whose obstacle rule is pinned to a numpy
restatement of the reference's (tests/test_obstacles_oracle.py)."""
import numpy as np
import pytest

import oracle
from conftest import assert_close, assert_rel, ulp32
from fltk_sph_ice_gb300 import FsphError, abi, rxPBDSPH, rxSPH, scenes

pytestmark = pytest.mark.gpu


def scene(solver="pbf"):
    """A block falling onto a rotated box and a sphere."""
    h = scenes.H_DEFAULT
    s = 0.5 * h
    box_max = [0.8, 0.8, 0.5]
    pos = scenes.lattice_block([0.25, 0.35, 0.12], (16, 12, 12), s, 0.01 * h, 9, 0)
    p = scenes.pbf_params(h, [0, 0, 0], box_max, pos.shape[0])
    p.eta, p.min_iter, p.max_iter = 0.0, 4, 4
    p.xsph_c, p.vort_eps = 0.0, 0.0
    if solver == "sph":
        p.solver = abi.SOLVER_WCSPH
        p.mass, p.gas_k, p.viscosity = 0.02, 3.0, 3.5 / scenes.REST_DENS
    vel = np.zeros_like(pos)
    vel[:, 1] = -1.5
    boxes = [((0.35, 0.18, 0.25), (0.08, 0.04, 0.15), (0.0, 30.0, 15.0))]
    spheres = [((0.55, 0.2, 0.25), 0.09)]
    return p, pos, vel, boxes, spheres


def with_obstacles(ps, boxes, spheres):
    for c, e, a in boxes:
        ps.SetBoxObstacle(c, e, a)
    for c, r in spheres:
        ps.SetSphereObstacle(c, r)


@pytest.mark.parametrize("solver", ["pbf", "sph"])
def test_obstacle_steps_match_oracle(gpu, solver):
    p, pos, vel, boxes, spheres = scene(solver)
    cls = rxPBDSPH if solver == "pbf" else rxSPH
    ps = cls(p)
    ps.Set(pos, vel)
    with_obstacles(ps, boxes, spheres)
    o = oracle.Oracle(p, pos.shape[0], threads=4)
    o.set(pos, vel)
    o.set_obstacles(boxes=boxes, spheres=spheres)
    dt = 0.0016 if solver == "pbf" else 0.001
    x0g = x0o = pos[:, :3].astype(np.float64)
    for k in range(40):
        ps.Update(dt)
        if solver == "pbf":
            o.pbf_step(dt, fixed_iters=4)
        else:
            o.sph_step(dt)
        xg, xo = ps.GetArrayVBO(abi.RX_POSITION)[:, :3], o.get("pos")[:, :3]
        if k < 3:
            assert_close(xg - x0g, xo - x0o, f"{solver} step {k + 1}: position change",
                         atol=ulp32(xo) + ulp32(x0o) + np.abs(x0g - x0o))
        x0g, x0o = xg.astype(np.float64), xo.astype(np.float64)
    # after the block has hit the obstacles: same state to the parity bar
    assert_rel(xg, xo, 1e-4, f"{solver}: positions after 40 steps")


def test_nothing_enters_the_obstacles(gpu):
    p, pos, vel, boxes, spheres = scene()
    p.max_iter, p.eta = 30, 1e-3
    ps = rxPBDSPH(p)
    ps.Set(pos, vel)
    with_obstacles(ps, boxes, spheres)
    from test_obstacles_oracle import euler
    touched = 0
    for _ in range(150):
        ps.Update(0.0016)
        x = ps.GetArrayVBO(abi.RX_POSITION)[:, :3].astype(np.float64)
        for c, e, a in boxes:
            cp = (x - c) @ euler(*a).T
            assert not ((np.abs(cp) - np.asarray(e) < -1e-5).all(1)).any(), "a particle inside the box"
            touched += int(((np.abs(cp) - np.asarray(e)) < 2e-3).all(1).sum())
        for c, r in spheres:
            d = np.linalg.norm(x - c, axis=1)
            assert (d > r - 1e-5).all(), "a particle inside the sphere"
            touched += int((d < r + 2e-3).sum())
    assert touched > 0  # the fluid reached the obstacles


def test_moving_sphere_obstacle(gpu):
    p, pos, vel, _, _ = scene()
    ps = rxPBDSPH(p)
    ps.Set(pos, np.zeros_like(pos))
    ps.SetSphereObstacle((0.1, 0.1, 0.1), 0.05)
    ps.MoveSphereObstacle(0, (0.2, 0.3, 0.1))
    assert np.allclose(ps.GetSphereObstaclePos(0), (0.3, 0.4, 0.2), atol=1e-6)
    c = ps.GetSphereObstaclePos(0)
    ps.Update(0.0016)
    x = ps.GetArrayVBO(abi.RX_POSITION)[:, :3]
    assert (np.linalg.norm(x - c, axis=1) > 0.05 - 1e-5).all()  # the sphere, moved into the block, cleared it
    with pytest.raises(FsphError):
        ps.MoveSphereObstacle(3, (0, 0, 0))
    for _ in range(9):  # ten spheres in all, the reference's MAX_SPHERE_NUM
        ps.SetSphereObstacle((0.0, 0.0, 0.0), 0.01)
    with pytest.raises(FsphError):
        ps.SetSphereObstacle((0.0, 0.0, 0.0), 0.01)
    ps.ClearObstacles()
    ps.Update(0.0016)

