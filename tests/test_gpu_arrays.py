"""SetArrayVBO / GetArrayVBO on a stepped state (rx_ps.h:253-262): the device
keeps the particles in cell order between steps; positions and velocities
set in particle order land in their particles' slots, and nothing else
moves.  Bars: arrays read back bit-exactly; a GetArrayVBO -> SetArrayVBO
round trip leaves the trajectory bit-identical (with and without the
warm-start history); a state set through SetArrayVBO steps like the same
state loaded with Set to FP32 rounding (the within-cell order, and so the
summation order, may differ)."""
import numpy as np
import pytest

from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes

pytestmark = pytest.mark.gpu


def _scene():
    sc = scenes.pbf_double_dam_break(block=(10, 10, 20))
    p = sc.params
    p.max_iter, p.min_iter = 6, 2
    return sc, p


def _stepped(p, sc, steps):
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    for _ in range(steps):
        ps.Update(sc.dt)
    return ps


def test_set_arrays_read_back_in_particle_order(gpu):
    sc, p = _scene()
    ps = _stepped(p, sc, 5)
    rng = np.random.default_rng(3)
    pos = ps.GetArrayVBO(abi.RX_POSITION)
    vel = ps.GetArrayVBO(abi.RX_VELOCITY)
    pos[:, :3] += rng.uniform(-1e-4, 1e-4, (sc.n, 3)).astype(np.float32)
    vel[:, :3] *= np.float32(0.5)
    ps.SetArrayVBO(abi.RX_POSITION, pos)
    ps.SetArrayVBO(abi.RX_VELOCITY, vel)
    assert np.array_equal(ps.GetArrayVBO(abi.RX_POSITION), pos)
    assert np.array_equal(ps.GetArrayVBO(abi.RX_VELOCITY), vel)
    ids = np.asarray(ps.GetArrayVBO(abi.FSPH_SORTED_ID)).reshape(-1)
    assert np.array_equal(np.sort(ids), np.arange(sc.n))  # still a permutation: the slots kept their particles
    ps.close()


def test_partial_range_leaves_the_rest(gpu):
    sc, p = _scene()
    ps = _stepped(p, sc, 3)
    before = ps.GetArrayVBO(abi.RX_POSITION)
    start, count = 100, 257
    new = before[start:start + count].copy()
    new[:, 1] += np.float32(0.01)
    ps.SetArrayVBO(abi.RX_POSITION, new, start, count)
    after = ps.GetArrayVBO(abi.RX_POSITION)
    assert np.array_equal(after[start:start + count], new)
    assert np.array_equal(np.delete(after, np.s_[start:start + count], 0),
                          np.delete(before, np.s_[start:start + count], 0))
    ps.close()


@pytest.mark.parametrize("warm", [0, 1])
def test_round_trip_leaves_the_trajectory(gpu, warm):
    """GetArrayVBO -> SetArrayVBO of positions and velocities around every
    step (the host round trip of a caller that owns the state) gives the
    same steps bit for bit as stepping without it, warm-start history
    included."""
    from fltk_sph_ice_gb300 import warmstart
    sc, p = _scene()
    p.warm_start = warm
    blob = warmstart.load_model()[0] if warm else None
    ctx = []
    for _ in range(2):
        ps = rxPBDSPH(p)
        if warm:
            ps.SetWarmStartModel(blob)
        ps.Set(sc.pos, sc.vel)
        ctx.append(ps)
    a, b = ctx
    for _ in range(6):
        a.Update(sc.dt)
        b.Update(sc.dt)
        b.SetArrayVBO(abi.RX_VELOCITY, b.GetArrayVBO(abi.RX_VELOCITY))
        b.SetArrayVBO(abi.RX_POSITION, b.GetArrayVBO(abi.RX_POSITION))
        assert a.last_stats.iterations == b.last_stats.iterations
    assert np.array_equal(a.GetArrayVBO(abi.RX_POSITION), b.GetArrayVBO(abi.RX_POSITION))
    assert np.array_equal(a.GetArrayVBO(abi.RX_VELOCITY), b.GetArrayVBO(abi.RX_VELOCITY))
    a.close()
    b.close()


def test_set_arrays_step_like_a_fresh_set(gpu):
    """A stepped context given (P, V) through SetArrayVBO, and a new context
    given (P, V) through Set, take the same next steps to FP32 rounding
    (plain solver: no warm-start history; bar 1e-5 of the field's range)."""
    sc, p = _scene()
    ps = _stepped(p, sc, 4)
    P = ps.GetArrayVBO(abi.RX_POSITION)
    V = ps.GetArrayVBO(abi.RX_VELOCITY)
    ps.SetArrayVBO(abi.RX_VELOCITY, V)
    ps.SetArrayVBO(abi.RX_POSITION, P)
    fresh = rxPBDSPH(p)
    fresh.Set(P, V)
    for _ in range(2):
        ps.Update(sc.dt)
        fresh.Update(sc.dt)
        assert abs(ps.last_stats.iterations - fresh.last_stats.iterations) <= 1
    x, y = ps.GetArrayVBO(abi.RX_POSITION)[:, :3], fresh.GetArrayVBO(abi.RX_POSITION)[:, :3]
    assert np.abs(x.astype(np.float64) - y).max() <= 1e-5 * np.abs(y).max()
    ps.close()
    fresh.close()


def test_set_arrays_keep_every_array_per_particle(gpu):
    """The warm-start history (step corrections, features) and the last
    step's results (density, lambda, vorticity, ...) still read back per
    particle after a SetArrayVBO, before and after a second one."""
    sc, p = _scene()
    p.collect_features = 1
    ps = _stepped(p, sc, 4)
    kinds = [abi.FSPH_FEATURES, abi.RX_STEP_CORRECTION, abi.RX_DENSITY, abi.RX_SCALING_FACTOR,
             abi.RX_VORTICITY, abi.RX_PREDICT_POS, abi.RX_CORRECTION]
    before = {k: ps.GetArrayVBO(k) for k in kinds}
    ps.SetArrayVBO(abi.RX_POSITION, ps.GetArrayVBO(abi.RX_POSITION))
    for k in kinds:
        assert np.array_equal(ps.GetArrayVBO(k), before[k]), k
    ps.SetArrayVBO(abi.RX_VELOCITY, ps.GetArrayVBO(abi.RX_VELOCITY))
    for k in kinds:
        assert np.array_equal(ps.GetArrayVBO(k), before[k]), k
    ps.close()
