"""Batched scenes (fsph_batch_*): every scene of a batch must step exactly as
the same scene stepped alone -- by the single-scene path and by the CPU
oracle -- under every launch configuration the autotuner can pick.

Bar: positions and velocities within 1e-5 in max|a-b| / max|b| per scene
after the stated steps (FP32; the batch re-sorts all scenes whenever one
needs a grid rebuild, so summation orders differ from a lone scene's)."""
import numpy as np
import pytest

import oracle
from conftest import assert_rel
from fltk_sph_ice_gb300 import FsphError, PBFBatch, abi, rxPBDSPH, scenes

pytestmark = pytest.mark.gpu

ITERS = 4


def small_set(count=6, seed=11):
    sc = scenes.batched_scenes(count=count, seed=seed, n_lo=512, n_hi=3000)
    for s in sc:
        s.params.min_iter = ITERS
        s.params.max_iter = ITERS
    return sc


def make_batch(sc):
    b = PBFBatch([s.params for s in sc], [s.n for s in sc], iterations=ITERS)
    b.set_particles(np.concatenate([s.pos for s in sc]), np.concatenate([s.vel for s in sc]))
    return b


def test_offsets_and_round_trip(gpu):
    sc = small_set()
    b = make_batch(sc)
    assert list(b.offsets) == list(np.concatenate([[0], np.cumsum([s.n for s in sc])]))
    x = b.get(abi.RX_POSITION)
    for k, s in enumerate(sc):
        np.testing.assert_array_equal(b.scene(x, k)[:, :3], s.pos[:, :3])


@pytest.mark.parametrize("nsteps", [1, 3])
def test_batch_matches_single_scenes(gpu, nsteps):
    sc = small_set()
    b = make_batch(sc)
    for _ in range(nsteps):
        b.step(sc[0].dt)
    xb, vb = b.get(abi.RX_POSITION), b.get(abi.RX_VELOCITY)
    for k, s in enumerate(sc):
        ps = rxPBDSPH(s.params)
        ps.Set(s.pos, s.vel)
        for _ in range(nsteps):
            ps.Update(s.dt)
        assert ps.LastStats().iterations == ITERS
        assert_rel(b.scene(xb, k)[:, :3], ps.GetArrayVBO(abi.RX_POSITION)[:, :3], 1e-5, f"scene {k} position")
        assert_rel(b.scene(vb, k)[:, :3], ps.GetArrayVBO(abi.RX_VELOCITY)[:, :3], 1e-4, f"scene {k} velocity")
        st = b.scene_stats(k)
        assert st.iterations == ITERS
        assert np.isfinite(st.density_error_one_sided) and st.status == abi.OK
        ps.close()


def test_batch_matches_oracle(gpu):
    sc = small_set(count=4, seed=12)
    b = make_batch(sc)
    b.step(sc[0].dt)
    xb = b.get(abi.RX_POSITION)
    db = b.get(abi.RX_DENSITY)
    for k, s in enumerate(sc):
        o = oracle.Oracle(s.params, s.n, threads=4)
        o.set(s.pos, s.vel)
        o.pbf_step(s.dt, fixed_iters=ITERS)
        assert_rel(b.scene(xb, k)[:, :3], o.get("pos")[:, :3], 1e-5, f"scene {k} position")
        assert_rel(b.scene(db, k), o.get("dens"), 1e-5, f"scene {k} density")


@pytest.mark.parametrize("block,lanes,skin", [(128, 1, 0.05), (256, 2, 0.1), (512, 4, 0.2), (256, 4, 0.05),
                                              (512, 1, 0.1), (128, 2, 0.2)])
def test_every_configuration_agrees(gpu, block, lanes, skin):
    sc = small_set(count=5, seed=13)
    ref = make_batch(sc)
    ref.set_config(256, 1, 0.05)
    b = make_batch(sc)
    b.set_config(block, lanes, skin)
    c = b.config
    assert (c.block, c.lanes) == (block, lanes) and abs(c.cell_skin - skin) < 1e-7
    for _ in range(2):
        ref.step(sc[0].dt)
        b.step(sc[0].dt)
    assert_rel(b.get(abi.RX_POSITION)[:, :3], ref.get(abi.RX_POSITION)[:, :3], 1e-5, "positions")


def test_autotune_restores_state_and_caches(gpu):
    sc = small_set(count=5, seed=14)
    b = make_batch(sc)
    b.step(sc[0].dt)
    x0 = b.get(abi.RX_POSITION)
    cfg, ms = b.autotune(sc[0].dt, steps=2)
    assert cfg.block in (128, 256, 512) and cfg.lanes in (1, 2, 4) and cfg.cell_skin in (
        np.float32(0.05), np.float32(0.1), np.float32(0.2))
    assert ms > 0.0
    np.testing.assert_array_equal(b.get(abi.RX_POSITION), x0)
    # the same scene set again: the cached winner, untimed
    b2 = make_batch(sc)
    cfg2, ms2 = b2.autotune(sc[0].dt, steps=2)
    assert ms2 == -1.0 and (cfg2.block, cfg2.lanes) == (cfg.block, cfg.lanes)
    # the tuned batch still steps like the default one
    ref = make_batch(sc)
    ref.step(sc[0].dt)
    ref.step(sc[0].dt)
    b.step(sc[0].dt)
    assert_rel(b.get(abi.RX_POSITION)[:, :3], ref.get(abi.RX_POSITION)[:, :3], 1e-5, "tuned vs default")


def test_empty_and_single_scenes(gpu):
    """Scenes without particles take no tiles and report zero error; a
    one-scene batch steps like the single-scene path."""
    sc = small_set(count=2, seed=15)
    empty = scenes.batched_scenes(count=1, seed=16, n_lo=512, n_hi=600)[0]
    params = [empty.params, sc[0].params, empty.params, sc[1].params]
    counts = [0, sc[0].n, 0, sc[1].n]
    for p in params:
        p.min_iter = p.max_iter = ITERS
    b = PBFBatch(params, counts, iterations=ITERS)
    b.set_particles(np.concatenate([sc[0].pos, sc[1].pos]), np.concatenate([sc[0].vel, sc[1].vel]))
    b.step(sc[0].dt)
    assert b.scene_stats(0).density_error_one_sided == 0.0 and b.scene_stats(2).density_error_max == 0.0
    x = b.get(abi.RX_POSITION)
    for k, s in ((1, sc[0]), (3, sc[1])):
        ps = rxPBDSPH(s.params)
        ps.Set(s.pos, s.vel)
        ps.Update(s.dt)
        assert_rel(b.scene(x, k)[:, :3], ps.GetArrayVBO(abi.RX_POSITION)[:, :3], 1e-5, f"scene {k}")
        ps.close()
    one = make_batch(sc[:1])
    one.step(sc[0].dt)
    ps = rxPBDSPH(sc[0].params)
    ps.Set(sc[0].pos, sc[0].vel)
    ps.Update(sc[0].dt)
    assert_rel(one.get(abi.RX_POSITION)[:, :3], ps.GetArrayVBO(abi.RX_POSITION)[:, :3], 1e-5, "one-scene batch")


def test_invalid_arguments(gpu):
    sc = small_set(count=2)
    with pytest.raises(FsphError):
        PBFBatch([s.params for s in sc], [s.n for s in sc], iterations=0)
    b = make_batch(sc)
    with pytest.raises(FsphError):
        b.set_config(100, 1, 0.05)
    with pytest.raises(FsphError):
        b.set_config(256, 3, 0.05)
    with pytest.raises(FsphError):
        b.set_config(256, 1, 0.9)
    bad = np.concatenate([s.pos for s in sc]).copy()
    bad[3, 1] = np.nan
    with pytest.raises(FsphError):
        b.set_particles(bad)
