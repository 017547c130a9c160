"""Checkpoint / resume: save -> load -> step is bit-identical to continuing
without the checkpoint (fsph_save_state / fsph_load_state), with every
piece of carried state live: the slot order, the learned warm start's
history and network, inlet lines mid-ring, deletion regions, a moved
sphere obstacle, boundary particles.  The reference's own checkpoint is
the particle file (OutputParticles / InputParticles, rx_ps.cpp:581-644),
which SaveCheckpoint writes beside the state with a JSON sidecar."""
import json

import numpy as np
import pytest

from fltk_sph_ice_gb300 import FsphError, abi, rxPBDSPH, rxSPH, scenes, warmstart

pytestmark = pytest.mark.gpu


def _pbf_scene(warm):
    sc = scenes.pbf_double_dam_break(block=(12, 12, 24))
    p = abi.FsphParams.from_buffer_copy(sc.params)
    p.max_particles = sc.n + 3000
    p.min_iter, p.max_iter = 2, 8
    p.warm_start = 1 if warm else 0
    ps = rxPBDSPH(p)
    if warm:
        blob, _ = warmstart.load_model()
        ps.SetWarmStartModel(blob)
    ps.Set(sc.pos, sc.vel)
    ps.SetSphereObstacle((0.3, 0.1, 0.15), 0.05)
    ps.SetBoxObstacle((0.5, 0.05, 0.1), (0.03, 0.03, 0.03), (0.0, 30.0, 0.0))
    ps.AddDeleteRegion((0.55, 0.0, 0.0), (0.6, 0.5, 0.3))
    ps.AddLine(pos1=(0.05, 0.3, 0.05), pos2=(0.05, 0.3, 0.2), vel=(0.4, 0.0, 0.0), up=(0.0, 1.0, 0.0), accum=2,
               span=3, spacing=2.0)
    return sc, ps


def _state(ps):
    return (ps.GetArrayVBO(abi.RX_POSITION), ps.GetArrayVBO(abi.RX_VELOCITY), ps.GetArrayVBO(abi.RX_ATTRIBUTE),
            ps.GetNumActiveParticles())


def _same(a, b):
    assert a[3] == b[3]
    for u, v in zip(a[:3], b[:3]):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("warm", [0, 1])
def test_pbf_resume_is_bit_identical(gpu, tmp_path, warm):
    sc, ps = _pbf_scene(warm)
    for step in range(25):
        ps.Update(sc.dt, step)
    ps.MoveSphereObstacle(0, (0.01, 0.0, 0.0))
    path = str(tmp_path / "ckpt.dat")
    ps.SaveCheckpoint(path, seed=1234)
    for step in range(25, 45):
        ps.Update(sc.dt, step)
    want = _state(ps)
    iters = ps.LastStats().iterations

    p2 = abi.FsphParams.from_buffer_copy(sc.params)  # different settings: the state carries its own
    p2.max_particles = sc.n
    fresh = rxPBDSPH(p2)
    assert fresh.LoadCheckpoint(path) == 1234
    assert fresh.GetParams().max_particles == sc.n + 3000
    for step in range(25, 45):
        fresh.Update(sc.dt, step)
    _same(_state(fresh), want)
    assert fresh.LastStats().iterations == iters
    side = json.load(open(path + ".json"))
    assert side["seed"] == 1234 and side["particles"] > sc.n


def test_wcsph_resume_is_bit_identical(gpu, tmp_path):
    sc = scenes.wcsph_dam_break(n_side=20)
    ps = rxSPH(sc.params)
    ps.Set(sc.pos, sc.vel)
    for _ in range(30):
        ps.Update(sc.dt)
    path = str(tmp_path / "w.state")
    ps.SaveState(path)
    for _ in range(20):
        ps.Update(sc.dt)
    want = _state(ps)
    fresh = rxSPH(sc.params)
    fresh.LoadState(path)
    for _ in range(20):
        fresh.Update(sc.dt)
    _same(_state(fresh), want)


def test_particle_file_round_trip(gpu, tmp_path):
    """The reference's particle file alone restores positions and velocities
    (the slot order is not in it, so later steps may differ in rounding)."""
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    ps = rxPBDSPH(sc.params)
    ps.Set(sc.pos, sc.vel)
    for _ in range(10):
        ps.Update(sc.dt)
    path = str(tmp_path / "p.dat")
    ps.OutputParticles(path)
    raw = open(path, "rb").read()
    assert len(raw) == 4 + 24 * sc.n and np.frombuffer(raw[:4], np.uint32)[0] == sc.n
    fresh = rxPBDSPH(sc.params)
    fresh.InputParticles(path)
    assert np.array_equal(fresh.GetArrayVBO(abi.RX_POSITION)[:, :3], ps.GetArrayVBO(abi.RX_POSITION)[:, :3])
    assert np.array_equal(fresh.GetArrayVBO(abi.RX_VELOCITY)[:, :3], ps.GetArrayVBO(abi.RX_VELOCITY)[:, :3])


def test_bad_state_files_leave_the_context_unchanged(gpu, tmp_path):
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    ps = rxPBDSPH(sc.params)
    ps.Set(sc.pos, sc.vel)
    ps.Update(sc.dt)
    path = tmp_path / "s.state"
    ps.SaveState(str(path))
    good = path.read_bytes()
    before = _state(ps)
    for bad in (good[: len(good) // 2], b"NOTSTATE" + good[8:], good[:40]):
        path.write_bytes(bad)
        with pytest.raises(FsphError) as e:
            ps.LoadState(str(path))
        assert e.value.status == abi.INVALID_ARG
    _same(_state(ps), before)
    with pytest.raises(FsphError):
        rxSPH(scenes.wcsph_dam_break(n_side=8).params).LoadState(str(tmp_path / "missing.state"))
    path.write_bytes(good)
    with pytest.raises(FsphError):  # a PBF state into a WCSPH context
        rxSPH(scenes.wcsph_dam_break(n_side=8).params).LoadState(str(path))
