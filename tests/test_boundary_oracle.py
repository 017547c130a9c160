"""The oracle's boundary-particle terms against an independent brute-force
numpy restatement of the reference formulas (CPU only).

  psi_b    = m / sum_b' m W(r_bb')                         rx_sph_pbd.cpp:1061-1090
  rho_i   += sum_b rho0 psi_b W(r_ib)                      rx_sph_pbd.cpp:728-748
  sd_i    += sum_b |(rho0 psi_b / m) grad W(r_ib) / rho0|^2  rx_sph_pbd.cpp:795-818
  lambda_b = -C_b / (sd_b + eps), rho_b and sd_b over fluid and boundary
             neighbours                                    rx_sph_pbd.cpp:825-913
  dp_i    += sum_b (lambda_i + lambda_b + s_corr_b) grad W(r_ib) / rho0,
             s_corr_b from (rho0 psi_b / m) W / W(dq)       rx_sph_pbd.cpp:977-1019
The reference's boundary code is compiled out by default (rx_sph.h:35); its
CPU version counts each boundary |grad C|^2 term twice (the neighbour vector
of rx_sph_pbd.cpp:731 is appended to again at :799) and finds a boundary
particle's fluid neighbours on the step-start positions (:833, :1714); the
oracle counts once and uses the current positions, as the reference's GPU
kernels do (rx_pbdsph_kernel.cu:577-735).  Bar: 1e-5 relative (float oracle
against double numpy)."""
import numpy as np

import oracle
from fltk_sph_ice_gb300 import abi, scenes


def kernels(h):
    aw = 315.0 / (64.0 * np.pi * h ** 9)
    ag = -45.0 / (np.pi * h ** 6)

    def W(r):
        return np.where(r <= h, aw * (h * h - r * r) ** 3, 0.0)

    def G(r):  # grad W = G(r) * d, d = x_i - x_j
        rr = np.maximum(r, 1e-300)
        return np.where((r <= h) & (r > 0), ag * (h - r) ** 2 / rr, 0.0)
    return W, G


def setup(seed=3):
    h = scenes.H_DEFAULT
    s = 0.5 * h
    bnd = scenes.box_surface([0.0, 0.0, 0.0], 6 * s, 0.3 * h)
    rng = np.random.default_rng(seed)
    n = 120
    pos = np.zeros((n, 4), np.float32)
    pos[:, 0] = rng.uniform(0.0, 6 * s, n)
    pos[:, 2] = rng.uniform(0.0, 6 * s, n)
    pos[:, 1] = 6 * s + rng.uniform(0.2 * h, 1.2 * h, n)
    p = scenes.pbf_params(h, [-1, -1, -1], [1, 1, 1], n)
    return pos, bnd, p


def pairs(a, b):
    d = a[:, None, :3].astype(np.float64) - b[None, :, :3].astype(np.float64)
    r = np.sqrt((d * d).sum(-1))
    return d, r


def test_boundary_terms_match_numpy():
    pos, bnd, p = setup()
    h, m, r0, eps = float(np.float32(p.h)), float(np.float32(p.mass)), float(np.float32(p.rest_dens)), float(p.epsilon)
    W, G = kernels(h)
    # psi_b
    _, rbb = pairs(bnd, bnd)
    psi = m / (m * W(rbb)).sum(1)
    o = oracle.Oracle(p, pos.shape[0])
    o.set_boundary(bnd)
    np.testing.assert_allclose(o.get_boundary("vol"), psi, rtol=1e-5)
    # fluid density and lambda
    dff, rff = pairs(pos, pos)
    dfb, rfb = pairs(pos, bnd)
    rho = (m * W(rff)).sum(1) + (r0 * psi[None, :] * W(rfb)).sum(1)
    gf = G(rff)[..., None] * dff / r0
    sd = (gf ** 2).sum(-1).sum(1) + (gf.sum(1) ** 2).sum(-1)
    gb = (r0 * psi / m)[None, :, None] * G(rfb)[..., None] * dfb / r0
    sd += (gb ** 2).sum(-1).sum(1)
    lam = -(rho / r0 - 1.0) / (sd + eps)
    d_o, l_o = o.lambda_pass(pos)
    np.testing.assert_allclose(d_o, rho, rtol=1e-5)
    assert np.abs(l_o - lam).max() <= 1e-5 * np.abs(lam).max()
    # boundary lambda
    dbf, rbf = pairs(bnd, pos)
    dbb, _ = pairs(bnd, bnd)
    rho_b = (m * W(rbf)).sum(1) + (r0 * psi[None, :] * W(rbb)).sum(1)
    sd_b = ((G(rbf)[..., None] * dbf / r0) ** 2).sum(-1).sum(1)
    sd_b += (((r0 * psi / m)[None, :, None] * G(rbb)[..., None] * dbb / r0) ** 2).sum(-1).sum(1)
    lam_b = -(rho_b / r0 - 1.0) / (sd_b + eps)
    lb_o = o.get_boundary("lambda")
    assert np.abs(lb_o - lam_b).max() <= 1e-5 * np.abs(lam_b).max()
    # position correction
    dt = 0.0016
    dq = p.ap_q * h
    wq = W(np.float64(dq))
    lam32, lamb32 = l_o.astype(np.float64), lb_o.astype(np.float64)
    sc = -p.ap_k * (W(rff) / wq) ** p.ap_n * dt * dt
    coef = lam32[:, None] + lam32[None, :] + sc
    dp = ((coef * G(rff))[..., None] * dff / r0).sum(1)
    scb = -p.ap_k * ((r0 * psi / m)[None, :] * W(rfb) / wq) ** p.ap_n * dt * dt
    coefb = lam32[:, None] + lamb32[None, :] + scb
    dp += ((coefb * G(rfb))[..., None] * dfb / r0).sum(1)
    o.L.fsph_orc_pbf_correction(o.h, oracle._vp(np.ascontiguousarray(pos)), oracle._vp(l_o.astype(np.float32)),
                                dt, oracle._vp(out := np.zeros((pos.shape[0], 4), np.float32)))
    assert np.abs(out[:, :3] - dp).max() <= 1e-5 * np.abs(dp).max()
    # the boundary matters in this configuration
    assert (r0 * psi[None, :] * W(rfb)).sum(1).max() > 0.1 * r0


def test_box_surface_counts_each_point_once():
    b = scenes.box_surface([0, 0, 0], 1.0, 0.1)
    m = 10
    assert b.shape[0] == (m + 1) ** 3 - (m - 1) ** 3
    assert np.unique(np.round(b[:, :3] * 1000).astype(np.int64), axis=0).shape[0] == b.shape[0]
