"""The oracle's analytic obstacles against an independent numpy restatement
of the reference's rule (CPU only): collisionPointBox / collisionPointSphere
(rx_cu_common.cu:748-831) as calCollisionSolidPB applies them
(rx_pbdsph_kernel.cu:863-911) -- a point inside a box, in the box's frame
rotated by EulerToMatrix (rx_sph_commons.h:185-210, degrees, pitch / yaw /
roll), moves onto the face nearest to it (ties in x, y, z order), a point
inside a sphere radially onto its surface; obstacles first, then the box
walls.  Bar: 1e-6 absolute (float oracle against double numpy, metres)."""
import numpy as np

import oracle
from fltk_sph_ice_gb300 import scenes


def euler(pitch, yaw, roll):
    p, y, r = np.radians([pitch, yaw, roll])
    cy, sy, cp, sp, cr, sr = np.cos(y), np.sin(y), np.cos(p), np.sin(p), np.cos(r), np.sin(r)
    cc, cs, sc, ss = cy * cr, cy * sr, sy * cr, sy * sr
    return np.array([[cc + sp * ss, cs - sp * sc, -sy * cp], [-cp * sr, cp * cr, -sp], [sc - sp * cs, ss + sp * cc, cy * cp]])


def project_numpy(x, boxes, spheres, lo, hi):
    x = np.array(x, np.float64)
    for cen, ext, ang in boxes:
        R = euler(*ang)
        cp = (x - cen) @ R.T
        t = np.abs(cp) - ext
        inside = (t < 0).all(1)
        a = -t
        ax = np.where((a[:, 0] <= a[:, 1]) & (a[:, 0] <= a[:, 2]), 0, np.where(a[:, 1] <= a[:, 2], 1, 2))
        rows = np.nonzero(inside)[0]
        cp[rows, ax[rows]] = np.where(cp[rows, ax[rows]] > 0, 1.0, -1.0) * np.asarray(ext)[ax[rows]]
        x = np.where(inside[:, None], cp @ R + cen, x)
    for cen, rad in spheres:
        l = x - cen
        ll = np.linalg.norm(l, axis=1)
        hit = (ll < rad) & (ll > 0)
        x = np.where(hit[:, None], cen + l * (rad / np.where(ll > 0, ll, 1.0))[:, None], x)
    return np.clip(x, lo, hi)


def test_obstacle_projection_matches_numpy():
    h = scenes.H_DEFAULT
    p = scenes.pbf_params(h, [0, 0, 0], [1.0, 0.8, 0.6], 10)
    boxes = [((0.3, 0.3, 0.3), (0.1, 0.05, 0.08), (20.0, 35.0, -10.0)), ((0.7, 0.4, 0.3), (0.06, 0.06, 0.06), (0, 0, 0))]
    spheres = [((0.5, 0.6, 0.3), 0.1)]
    rng = np.random.default_rng(5)
    n = 20000
    x = np.zeros((n, 4), np.float32)
    x[:, :3] = rng.uniform([-0.05, -0.05, -0.05], [1.05, 0.85, 0.65], (n, 3))
    o = oracle.Oracle(p, n)
    o.set_obstacles(boxes=boxes, spheres=spheres)
    got = o.project(x)[:, :3].astype(np.float64)
    r = float(np.float32(p.particle_radius))
    lo = np.array([r, r, r])
    hi = np.array([1.0, 0.8, 0.6]) - r
    want = project_numpy(x[:, :3].astype(np.float64), boxes, spheres, lo, hi)
    moved = np.abs(want - x[:, :3]).max(1) > 0
    assert moved.sum() > 1000  # many points were inside an obstacle or outside the walls
    assert np.abs(got - want).max() < 1e-6, np.abs(got - want).max()
    # nothing is left inside an obstacle
    for cen, ext, ang in boxes:
        cp = (got - cen) @ euler(*ang).T
        assert not ((np.abs(cp) - np.asarray(ext) < -1e-6).all(1)).any()
    for cen, rad in spheres:
        assert (np.linalg.norm(got - cen, axis=1) > rad - 1e-6).all()
