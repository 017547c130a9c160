"""The grid build's two sorts give the same slot order: the LSD radix sort of
the 64-bit keys (cell << 32 | previous slot), grid_sort = 1, against the
counting sort with per-cell ordering, grid_sort = 0.  Same order means
bit-identical steps, in-loop grid rebuilds included (the reference sorts
with thrust::sort_by_key, rx_cu_funcs.cu:250-260)."""
import numpy as np
import pytest

from fltk_sph_ice_gb300 import abi, rxPBDSPH, rxSPH, scenes

pytestmark = pytest.mark.gpu


def _run(cls, sc, p, sort, steps):
    q = abi.FsphParams.from_buffer_copy(p)
    q.grid_sort = sort
    ps = cls(q)
    ps.Set(sc.pos, sc.vel)
    builds = 0
    for _ in range(steps):
        ps.Update(sc.dt)
        builds += ps.LastStats().grid_builds
    return ps.GetArrayVBO(abi.RX_POSITION), ps.GetArrayVBO(abi.RX_VELOCITY), builds


@pytest.mark.parametrize("graph", [0, 1])
def test_radix_and_counting_sorts_step_identically_pbf(gpu, graph):
    sc = scenes.pbf_double_dam_break(block=(24, 24, 48))
    p = sc.params
    p.use_graph = graph
    p.min_iter, p.max_iter = 2, 8
    x0, v0, b0 = _run(rxPBDSPH, sc, p, 0, 40)
    x1, v1, b1 = _run(rxPBDSPH, sc, p, 1, 40)
    assert b0 == b1 and b0 > 40  # in-loop rebuilds happened
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)


def test_radix_and_counting_sorts_step_identically_wcsph(gpu):
    sc = scenes.wcsph_dam_break(n_side=24)
    x0, v0, _ = _run(rxSPH, sc, sc.params, 0, 20)
    x1, v1, _ = _run(rxSPH, sc, sc.params, 1, 20)
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)


def test_radix_sort_at_262k(gpu):
    """The 262,144-particle PBF dam (64^3 lattice): several radix passes
    over a large cell table."""
    sc = scenes.pbf_dam_break(n_side=64)
    p = sc.params
    p.min_iter = p.max_iter = 4
    x0, _, _ = _run(rxPBDSPH, sc, p, 0, 3)
    x1, _, _ = _run(rxPBDSPH, sc, p, 1, 3)
    assert np.array_equal(x0, x1)


def test_grid_sort_is_validated(gpu):
    p = scenes.pbf_double_dam_break(block=(8, 8, 8)).params
    p.grid_sort = 2
    with pytest.raises(abi.FsphError) as e:
        rxPBDSPH(p)
    assert e.value.status == abi.INVALID_ARG
