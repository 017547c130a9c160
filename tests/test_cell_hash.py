"""Cell indices under the reference's own grid rules.

The reference has two grids: its CPU grid (rxNNGrid::Setup / CalGridHash,
rx_nnsearch.h:174-199, 578-599) and its GPU grid (setupCells,
rx_sph_pbd_gpu.cpp:1986-2011, with calcGridPos / calcGridHash,
rx_cu_common.cu:121-144).  A numpy restatement of both is pinned here to the
reference's compiled CPU grid (CPU, no GPU); the GPU entry point
fsph_reference_cell_hash must then equal both bit for bit.  The GPU rule is
float arithmetic that numpy float32 reproduces exactly (IEEE subtract and
divide, then floor)."""
import math

import numpy as np
import pytest

import oracle
from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes


def reference_grid(p, rule):
    """Geometry of the reference's grid over the box grown by 1 %
    (rx_sph_pbd.cpp:188-196), in the reference's order of operations."""
    lo = [p.box_min[a] - 0.5 * 0.01 * (p.box_max[a] - p.box_min[a]) for a in range(3)]
    hi = [lo[a] + (p.box_max[a] - p.box_min[a]) * (1.0 + 0.01) for a in range(3)]
    ws = [hi[a] - lo[a] for a in range(3)]
    h = float(np.float32(p.h))
    m_axis = max(ws)
    d = int(math.log(m_axis / h) / math.log(2.0) + 0.5)
    cw = m_axis / int(math.pow(2.0, d) + 0.5)
    if rule == 0:
        g = [int(math.pow(2.0, int(math.log(w / cw) / math.log(2.0) + 0.5)) + 0.5) for w in ws]
    else:
        g = [int(w / cw) + 1 for w in ws]
    return np.array(lo), cw, np.array(g)


def cell_hash_numpy(p, pos4, rule):
    lo, cw, g = reference_grid(p, rule)
    x = np.asarray(pos4, np.float32)[:, :3]
    if rule == 0:
        c = np.trunc((x.astype(np.float64) - lo) / cw)
    else:
        c = np.floor((x - lo.astype(np.float32)) / np.float32(cw))
    c = np.clip(c, 0, g - 1).astype(np.int64)
    return ((c[:, 2] * g[1] + c[:, 1]) * g[0] + c[:, 0]).astype(np.uint32), g, cw


def probe_positions(p, seed=7):
    """Particles of a dam scene, points on cell faces of both grids, and
    points outside the simulation range on every side."""
    sc = scenes.pbf_double_dam_break(block=(12, 12, 24))
    pts = [sc.pos[:, :3]]
    rng = np.random.default_rng(seed)
    for rule in (0, 1):
        lo, cw, g = reference_grid(p, rule)
        k = rng.integers(0, g + 1, size=(4000, 3))
        pts.append((lo + k * cw).astype(np.float32))
        pts.append((lo + k * cw + rng.choice([-1e-7, 1e-7], size=(4000, 3))).astype(np.float32))
    bmin, bmax = np.array(p.box_min), np.array(p.box_max)
    pts.append(rng.uniform(bmin - 0.2 * (bmax - bmin), bmax + 0.2 * (bmax - bmin), size=(4000, 3)).astype(np.float32))
    x = np.concatenate(pts).astype(np.float32)
    out = np.zeros((x.shape[0], 4), np.float32)
    out[:, :3] = x
    return sc, out


@pytest.fixture(scope="module")
def ref_lib():
    if oracle.ref_lib() is None:
        pytest.skip("reference CPU code not built")
    return oracle.ref_lib()


def test_numpy_cpu_rule_equals_reference_grid(ref_lib):
    sc = scenes.pbf_double_dam_break(block=(12, 12, 24))
    p = sc.params
    _, x = probe_positions(p)
    ref = oracle.RefSolver(p, x.shape[0], "pbf")
    got, ncell = ref.cell_hash(x)
    want, g, cw = cell_hash_numpy(p, x, 0)
    assert ncell == int(np.prod(g))
    assert np.array_equal(got, want)
    lo, _, _ = reference_grid(p, 0)
    s = ref.scalars()
    assert np.array_equal(s[7:10], lo)  # the simulation range's corner, bit for bit


def test_cpu_and_gpu_grids_differ():
    """The two reference grids disagree (power-of-two axis counts vs
    floor(L/cw) + 1), so the rule has to be named."""
    p = scenes.pbf_double_dam_break(block=(12, 12, 24)).params
    g0 = reference_grid(p, 0)[2]
    g1 = reference_grid(p, 1)[2]
    assert not np.array_equal(g0, g1)


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [0, 1])
def test_gpu_cell_hash_bit_exact(gpu, ref_lib, rule):
    sc = scenes.pbf_double_dam_break(block=(12, 12, 24))
    p = sc.params
    _, x = probe_positions(p)
    ps = rxPBDSPH(p)
    got, g, cw = ps.CalGridHash(x, rule)
    want, gw, cww = cell_hash_numpy(p, x, rule)
    assert np.array_equal(g, gw), (g, gw)
    assert cw == cww, (cw, cww)
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, (bad.size, bad[:5], got[bad[:5]], want[bad[:5]], x[bad[:5]])
    if rule == 0:
        ref, _ = oracle.RefSolver(p, x.shape[0], "pbf").cell_hash(x)
        bad = np.nonzero(got != ref)[0]
        assert bad.size == 0, (bad.size, bad[:5], got[bad[:5]], ref[bad[:5]], x[bad[:5]])


@pytest.mark.gpu
def test_gpu_cell_hash_on_stepped_state(gpu, ref_lib):
    """The cell hash of a stepped state (particles on the walls included)."""
    sc = scenes.pbf_double_dam_break(block=(16, 16, 32))
    ps = rxPBDSPH(sc.params)
    ps.Set(sc.pos, sc.vel)
    for _ in range(20):
        ps.Update(sc.dt)
    x = ps.GetArrayVBO(abi.RX_POSITION)
    got, _, _ = ps.CalGridHash(x, 0)
    ref, _ = oracle.RefSolver(sc.params, sc.n, "pbf").cell_hash(x)
    assert np.array_equal(got, ref)
    got1, _, _ = ps.CalGridHash(x, 1)
    assert np.array_equal(got1, cell_hash_numpy(sc.params, x, 1)[0])
