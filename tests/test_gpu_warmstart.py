"""Warm start of the PBF iterations on the GPU: the plumbing (step
corrections, features, both warm-start modes) and the gain of the trained
network committed in fltk_sph_ice_gb300/models.

A warm start only moves the point the iterations start from: every step
must still reach the same density-error tolerance, and the velocity and
position of a step follow from where the iterations stop."""
import ctypes
import os

import numpy as np
import pytest

from conftest import assert_rel
from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes, warmstart

pytestmark = pytest.mark.gpu


def make(block=(16, 16, 32), mode=0, collect=0, seed=3):
    sc = scenes.pbf_double_dam_break(block=block, seed=seed)
    p = sc.params
    p.clamp_constraint, p.eta, p.max_iter = 1, 1e-3, 300
    p.warm_start, p.collect_features = mode, collect
    return sc, p


def run(sc, p, steps, blob=None):
    ps = rxPBDSPH(p)
    if blob is not None:
        assert ps.L.fsph_set_warm_start_model(ps.handle, blob.ctypes.data_as(ctypes.c_void_p)) == abi.OK
    ps.Set(sc.pos, sc.vel)
    its, errs = [], []
    for _ in range(steps):
        ps.Update(sc.dt)
        its.append(ps.last_stats.iterations)
        errs.append(ps.last_stats.density_error_one_sided)
    return ps, np.array(its), np.array(errs)


def test_step_correction_and_features(gpu):
    sc, p = make(collect=1)
    ps, its, errs = run(sc, p, 3)
    x_before = ps.GetArrayVBO(abi.RX_POSITION)
    v_before = ps.GetArrayVBO(abi.RX_VELOCITY)
    feats = ps.GetArrayVBO(abi.FSPH_FEATURES)
    assert feats.shape == (sc.n, abi.MLP_FEATURES) and np.isfinite(feats).all()
    # features 9-11 are the last step's correction over h
    d_last = ps.GetArrayVBO(abi.RX_STEP_CORRECTION)[:, :3]
    assert_rel(feats[:, 9:12], d_last / p.h, 1e-6, "correction feature")
    ps.Update(sc.dt)
    x_after = ps.GetArrayVBO(abi.RX_POSITION)
    d = ps.GetArrayVBO(abi.RX_STEP_CORRECTION)[:, :3]
    # x_after = walls(x + dt (v + dt g)) + D: away from the walls, the prediction is unclipped
    g = np.array(p.gravity)
    pred = x_before[:, :3] + sc.dt * (v_before[:, :3] + sc.dt * g)
    lo = np.array(p.box_min) + p.particle_radius + 1e-4
    hi = np.array(p.box_max) - p.particle_radius - 1e-4
    inside = ((pred > lo) & (pred < hi)).all(1)
    assert inside.mean() > 0.5
    np.testing.assert_allclose(x_after[inside, :3], pred[inside] + d[inside], rtol=0, atol=2e-6)


def features_numpy(x, v, dens, lam, dstep, p, dt):
    """The end-of-step features restated by brute force over all pairs (FP64)."""
    h, r0, m = float(p.h), float(p.rest_dens), float(p.mass)
    aw = 315.0 / (64.0 * np.pi * h ** 9)
    ag = -45.0 / (np.pi * h ** 6)
    X, V = x[:, :3].astype(np.float64), v[:, :3].astype(np.float64)
    d = X[:, None, :] - X[None, :, :]                     # x_i - x_j
    r = np.sqrt((d * d).sum(-1))
    inside = r * r < h * h
    cnt = np.maximum(inside.sum(1), 1)
    ds = d - dt * (V[None, :, :] - V[:, None, :])        # x_ij + dt (v_i - v_j)
    rs = np.sqrt((ds * ds).sum(-1))
    qs = np.maximum(h * h - rs * rs, 0.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        gs = np.where((rs > 0) & (rs < h), ag * (h - rs) ** 2 / rs, 0.0)
    f = np.zeros((x.shape[0], abi.MLP_FEATURES))
    f[:, 0] = dens / r0 - 1.0
    f[:, 1] = lam * r0 * h * h
    f[:, 2] = inside.sum(1) / 33.0
    f[:, 3:6] = -(inside[..., None] * d).sum(1) / h / cnt[:, None]
    f[:, 6:9] = V * dt / h
    f[:, 9:12] = dstep[:, :3] / h
    f[:, 12] = m / r0 * aw * (qs ** 3).sum(1) - 1.0
    f[:, 13:16] = m / r0 * h * (gs[..., None] * ds).sum(1)
    # poly6-weighted means over the neighbours, self excluded
    w = np.where(r > 0, np.maximum(h * h - r * r, 0.0) ** 3, 0.0)
    nw = w.sum(1)
    has = nw > 0
    inw = np.where(has, 1.0 / np.where(has, nw, 1.0), 0.0)
    f[:, 16] = np.where(has, (w @ dens.astype(np.float64)) * inw / r0 - 1.0, 0.0)
    f[:, 17:20] = (w @ V) * inw[:, None] * dt / h
    f[:, 20:23] = (w @ dstep[:, :3].astype(np.float64)) * inw[:, None] / h
    return f


def test_features_match_numpy(gpu):
    """Every feature against a brute-force restatement, on a state where the
    velocity is the one the feature pass saw (XSPH and vorticity off)."""
    sc, p = make(block=(10, 8, 20), collect=1, seed=5)
    p.xsph_c, p.vort_eps = 0.0, 0.0
    ps, _, _ = run(sc, p, 25)
    f = ps.GetArrayVBO(abi.FSPH_FEATURES).reshape(sc.n, abi.MLP_FEATURES)
    ref = features_numpy(ps.GetArrayVBO(abi.RX_POSITION), ps.GetArrayVBO(abi.RX_VELOCITY),
                         ps.GetArrayVBO(abi.RX_DENSITY), ps.GetArrayVBO(abi.RX_SCALING_FACTOR),
                         ps.GetArrayVBO(abi.RX_STEP_CORRECTION), p, sc.dt)
    for k in range(abi.MLP_FEATURES):
        scale = max(np.abs(ref[:, k]).max(), 1e-3)
        err = np.abs(f[:, k] - ref[:, k]).max() / scale
        assert err < 2e-3, (k, err)


def test_unknown_warm_start_mode_rejected(gpu):
    sc, p = make(mode=2)
    with pytest.raises(abi.FsphError) as e:
        rxPBDSPH(p)
    assert e.value.status == abi.INVALID_ARG


def test_learned_warm_start_needs_a_model(gpu):
    sc, p = make(mode=abi.WARM_LEARNED)
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    with pytest.raises(abi.FsphError) as e:
        ps.Update(sc.dt)
    assert e.value.status == abi.UNSUPPORTED


@pytest.mark.skipif(not os.path.isfile(warmstart.DEFAULT_MODEL), reason="no trained model committed yet")
def test_trained_network_reduces_iterations(gpu):
    """What the trained network gains over the plain method on a held-out
    scene (seed and block size not in the training rollouts): fewer
    iterations per step at the same tolerance."""
    blob, meta = warmstart.load_model()
    block = (28, 24, 56)
    sc0, p0 = make(block=block, mode=0, seed=77)
    _, its0, err0 = run(sc0, p0, 120)
    sc1, p1 = make(block=block, mode=abi.WARM_LEARNED, seed=77)
    _, its1, err1 = run(sc1, p1, 120, blob=blob)
    m0, m1 = its0[40:].mean(), its1[40:].mean()
    print(f"plain {m0:.1f} iterations/step, learned warm start {m1:.1f} (steps 40-120)")
    assert (err1 <= p1.eta * (1 + 1e-6)).all()
    assert m1 < 0.8 * m0
