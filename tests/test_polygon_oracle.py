"""Triangle-mesh obstacles: a numpy restatement of the reference's GPU rule
pins the oracle's (CPU, no GPU).

The rule (rxPBDSPH_GPU::setPolysToCell, rx_sph_pbd_gpu.cpp:2051-2200;
pbdsphIntegrateWithPolygon / calCollisionPolygonPB, rx_pbdsph_kernel.cu:
916-1030; intersectSegmentTriangle, rx_cu_common.cu:891-975): triangles are
binned into the cells of the reference's GPU grid they intersect; a segment
x0 -> x1 meets the triangles of the cells of x0 and then of x1, each in
ascending index; a crossing from the front side puts x1 back on that side
and removes the velocity component into the triangle.  Float32, one
rounding per operation, so the comparison is bit for bit."""
import numpy as np
import pytest

import oracle
from fltk_sph_ice_gb300 import scenes
from test_cell_hash import reference_grid

F = np.float32


def tri_cube_overlap(v):
    """separating axes, triangle v (3, 3) against [-0.5, 0.5]^3 (Akenine-Moeller 2001)"""
    if (v.min(0) > 0.5).any() or (v.max(0) < -0.5).any():
        return False
    e = np.roll(v, -1, axis=0) - v
    for k in range(3):
        for a in range(3):
            ax = np.zeros(3)
            ax[(a + 1) % 3] = -e[k][(a + 2) % 3]
            ax[(a + 2) % 3] = e[k][(a + 1) % 3]
            q = v @ ax
            r = 0.5 * np.abs(ax).sum()
            if q.min() > r or q.max() < -r:
                return False
    n = np.cross(e[0], e[1])
    return abs(n @ v[0]) <= 0.5 * np.abs(n).sum()


def bin_triangles(p, V, T):
    lo, cw, g = reference_grid(p, 1)
    L = float(F(cw))
    cells = {}
    for i, t in enumerate(T):
        P = V[t].astype(np.float64)
        b0 = (P.min(0) - lo) / L
        b1 = (P.max(0) - lo) / L
        l0 = np.clip(np.trunc(np.clip(b0, -1, g)).astype(int), 0, g - 1)
        h0 = np.clip(np.trunc(np.clip(b1, -1, g)).astype(int), 0, g - 1)
        for x in range(l0[0], h0[0] + 1):
            for y in range(l0[1], h0[1] + 1):
                for z in range(l0[2], h0[2] + 1):
                    cen = lo + (np.array([x, y, z]) + 0.5) * L
                    if tri_cube_overlap((P - cen) / L):
                        cells.setdefault((z * g[1] + y) * g[0] + x, []).append(i)
    return cells, lo.astype(F), F(cw), g


def _dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def _cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], F)


def _unit(a):
    l = np.sqrt(_dot(a, a))
    return np.array([a[0] / l, a[1] / l, a[2] / l], F)


def seg_tri(P0, P1, V0, V1, V2):
    u, v = V1 - V0, V2 - V0
    c = _cross(u, v)
    if _dot(c, c) == 0:
        return -1, None, None
    n = _unit(c)
    d = P1 - P0
    a = _dot(n, P0 - V0)
    b = _dot(n, d)
    if float(abs(b)) < 1e-10:
        return (2 if a == 0 else 0), None, None
    r = -a / b
    if r < 0 or abs(a) > abs(b) or b > 0:
        return 0, None, None
    I = P0 + d * r
    uu, uv, vv = _dot(u, u), _dot(u, v), _dot(v, v)
    w = I - V0
    wu, wv = _dot(w, u), _dot(w, v)
    D = uv * uv - uu * vv
    s = (uv * wv - vv * wu) / D
    if s < 0 or s > 1:
        return 0, None, None
    t = (uv * wu - uu * wv) / D
    if t < 0 or s + t > 1:
        return 0, None, None
    return 1, I, n


def collide_numpy(p, V, T, x0, x1, v, dt):
    V = np.asarray(V, F)
    cells, org, cw, g = bin_triangles(p, V, T)
    dt = F(dt)
    x1, v = np.array(x1, F, copy=True), np.array(v, F, copy=True)

    def cell(x):
        f = np.floor((x[:3] - org) / cw)
        k = np.clip(np.clip(f, -1, g).astype(int), 0, g - 1)
        return (k[2] * g[1] + k[1]) * g[0] + k[0]

    hits = 0
    for i in range(x0.shape[0]):
        a, b, w = x0[i, :3].astype(F), x1[i, :3], v[i, :3]
        for c in (cell(a), cell(b)):
            for t in cells.get(c, []):
                st, cp, n = seg_tri(a, b, V[T[t][0]], V[T[t][1]], V[T[t][2]])
                if st != 1:
                    continue
                hits += 1
                dd = np.sqrt(_dot(b - cp, b - cp))
                n = _unit(n)
                vr = (n * F(-1)) * _dot(n, w)
                l = np.sqrt(_dot(b - a, b - a))
                b = cp + vr * ((dt * dd) / l)
                w = w + vr
        x1[i, :3], v[i, :3] = b, w
    return x1, v, hits


def ramp_mesh(p):
    """a tilted ramp of two triangles across the box (front side up) and a
    small closed box of 12 triangles"""
    lo, hi = np.array(p.box_min), np.array(p.box_max)
    e = hi - lo
    y0, y1 = lo[1] + 0.15 * e[1], lo[1] + 0.45 * e[1]
    V = [[lo[0] + 0.05 * e[0], y1, lo[2] + 0.05 * e[2]], [lo[0] + 0.95 * e[0], y0, lo[2] + 0.05 * e[2]],
         [lo[0] + 0.95 * e[0], y0, lo[2] + 0.95 * e[2]], [lo[0] + 0.05 * e[0], y1, lo[2] + 0.95 * e[2]]]
    T = [[0, 2, 1], [0, 3, 2]]
    c = lo + np.array([0.6, 0.7, 0.5]) * e
    s = 0.06 * e.min()
    for k in range(8):
        V.append(list(c + s * np.array([(k & 1) * 2 - 1, (k >> 1 & 1) * 2 - 1, (k >> 2 & 1) * 2 - 1])))
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    for q in quads:
        a, b, cc, d = (4 + k for k in q)
        T += [[a, b, cc], [a, cc, d]]
    return np.array(V, np.float64), np.array(T, np.int32)


def segments(p, V, T, n=3000, seed=11):
    """segments ending behind the ramp, crossing its plane, and random ones"""
    rng = np.random.default_rng(seed)
    lo, hi = np.array(p.box_min), np.array(p.box_max)
    Vf = V.astype(F).astype(np.float64)
    x0 = rng.uniform(lo, hi, (n, 3))
    t = rng.uniform(0, 1, (n, 2))
    on = Vf[0] + t[:, :1] * (Vf[1] - Vf[0]) + t[:, 1:] * (Vf[3] - Vf[0])
    m = n // 2
    up = np.cross(Vf[3] - Vf[0], Vf[1] - Vf[0])  # the triangles' front side
    up /= np.linalg.norm(up)
    x0[:m] = on[:m] + up * rng.uniform(1e-4, 0.02, (m, 1))
    d = rng.normal(0, 0.02, (n, 3))
    d[:m] = -up * rng.uniform(0.0, 0.04, (m, 1)) + rng.normal(0, 0.005, (m, 3))
    x1 = x0 + d
    v = d / 0.0016
    pad = lambda a: np.concatenate([a, np.zeros((n, 1))], 1).astype(F)  # noqa: E731
    return pad(x0), pad(x1), pad(v)


@pytest.fixture(scope="module")
def case():
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    V, T = ramp_mesh(sc.params)
    x0, x1, v = segments(sc.params, V, T)
    return sc.params, V, T, x0, x1, v


def test_numpy_rule_hits_and_misses(case):
    p, V, T, x0, x1, v = case
    y1, w, hits = collide_numpy(p, V, T, x0, x1, v, 0.0016)
    assert hits > 500  # half of the segments were aimed through the ramp
    moved = np.any(y1 != x1, axis=1)
    assert moved.sum() >= 500 and moved.sum() < x0.shape[0]
    up = np.cross(V[3] - V[0], V[1] - V[0])
    up /= np.linalg.norm(up)
    side = (y1[:1500, :3] - V[0]) @ up
    assert (side[moved[:1500]] > -1e-6).all()  # the deflected ones stay in front


def test_oracle_equals_numpy_rule(case):
    p, V, T, x0, x1, v = case
    want_x, want_v, _ = collide_numpy(p, V, T, x0, x1, v, 0.0016)
    o = oracle.Oracle(p, 8, threads=1)
    o.set_polygons(V, T)
    got_x, got_v = o.polygon_collide(x0, x1, v, 0.0016)
    assert np.array_equal(got_x, want_x)
    assert np.array_equal(got_v, want_v)


def test_binning_matches_brute_force_superset(case):
    """every (cell, triangle) the table holds overlaps the triangle's bounding
    box of cells, and a triangle through a cell centre is always binned there"""
    p, V, T, _, _, _ = case
    cells, org, cw, g = bin_triangles(p, V.astype(F), T)
    assert sum(len(c) for c in cells.values()) >= len(T)
    for t in range(len(T)):
        ctr = V[T[t]].astype(F).astype(np.float64).mean(0)
        k = np.clip(np.floor((ctr - org) / float(cw)).astype(int), 0, g - 1)
        assert t in cells[(k[2] * g[1] + k[1]) * g[0] + k[0]]
