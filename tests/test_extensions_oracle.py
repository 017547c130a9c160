"""The oracle's XSPH, vorticity-confinement and clamped-constraint terms
against an independent brute-force numpy restatement (CPU only).

These three terms have no CPU code in the reference to pin them against:
  XSPH      v_i + c sum_j (m / rho_j)(v_j - v_i) W(r_ij), r_ij <= h, self
            included (its term is zero): the reference's GPU kernel
            xsphVisocosity / calXsphViscosityCell (rx_pbdsph_kernel.cu:1090-1162),
            disabled at rx_sph_pbd_gpu.cpp:926-927;
  vorticity Macklin & Mueller 2013 ("Position Based Fluids", eq. 15-16, cited
            at rx_sph.h:1281; the reference has only the flag, rx_ps.h:161,238),
            with the curl weighted by the neighbour volume V_j = m / rho_j
            (the paper's eq. 15 leaves V_j to its eps; without it the
            configured eps = 1e-4 drives the dam breaks unstable):
              w_i   = sum_j V_j (v_j - v_i) x grad_j W(x_i - x_j),  grad_j W = -grad_i W
              eta_i = sum_j (m / rho_j)(|w_j| - |w_i|) grad_i W(x_i - x_j)
              f_i   = eps (eta_i / |eta_i|) x w_i, applied as an acceleration:
              v_i  <- v_i(after XSPH) + dt f_i
  clamp     the unilateral constraint of the same paper, C_i = max(rho_i/rho0 - 1, 0),
            in lambda_i = -C_i / (sum_k |grad_k C_i|^2 + eps) with the k = i term
            (rx_sph_pbd.cpp:699-914 for everything but the max).
Bars: 1e-5 relative to the field's largest magnitude (float oracle against
double numpy), and element-wise 1e-4 relative on every entry above 1 % of it
(plus one FP32 ulp where the compared value is a difference of stored results).
"""
import numpy as np

import oracle
from conftest import assert_close, ulp32
from fltk_sph_ice_gb300 import abi, scenes


def kernels(h):
    aw = 315.0 / (64.0 * np.pi * h ** 9)
    ag = -45.0 / (np.pi * h ** 6)

    def W(r):
        return np.where(r <= h, aw * (h * h - r * r) ** 3, 0.0)

    def G(r):  # grad_i W(x_i - x_j) = G(r) (x_i - x_j)
        rr = np.maximum(r, 1e-300)
        return np.where((r <= h) & (r > 0), ag * (h - r) ** 2 / rr, 0.0)
    return W, G


def state(seed=11, dims=(8, 7, 6)):
    """A jittered h/2 lattice block with a swirling velocity field and
    densities scattered around rho0."""
    h = scenes.H_DEFAULT
    s = 0.5 * h
    pos = scenes.lattice_block([0.1, 0.1, 0.1], dims, s, 0.2 * h, seed, 0)
    n = pos.shape[0]
    rng = np.random.default_rng(seed)
    c = pos[:, :3].mean(0)
    vel = np.zeros_like(pos)
    vel[:, 0] = -(pos[:, 1] - c[1]) * 3.0 + rng.normal(0, 0.05, n)
    vel[:, 1] = (pos[:, 0] - c[0]) * 3.0 + rng.normal(0, 0.05, n)
    vel[:, 2] = rng.normal(0, 0.1, n)
    dens = (scenes.REST_DENS * (1.0 + rng.uniform(-0.05, 0.05, n))).astype(np.float32)
    p = scenes.pbf_params(h, [0, 0, 0], [1, 1, 1], n)
    p.xsph_c, p.vort_eps = 0.01, 1e-4
    return pos, vel, dens, p


def pairs(x):
    d = x[:, None, :3].astype(np.float64) - x[None, :, :3].astype(np.float64)
    r = np.sqrt((d * d).sum(-1))
    return d, r


def xsph_vorticity_numpy(pos, vel, dens, p, dt, bounds=False):
    """Velocity after XSPH + confinement, and omega.  bounds=True also
    returns first-order bounds of the change each result sees when every
    pair term carries a relative error delta = 32 eps32 (FP32 evaluation and
    accumulation of ~40 terms): (d_velocity, d_omega) per particle."""
    h, m = float(np.float32(p.h)), float(np.float32(p.mass))
    c, eps = float(np.float32(p.xsph_c)), float(np.float32(p.vort_eps))
    W, G = kernels(h)
    d, r = pairs(pos)
    v = vel[:, :3].astype(np.float64)
    rho = dens.astype(np.float64)
    vij = v[None, :, :] - v[:, None, :]                       # v_j - v_i
    inside = r <= h
    wgt = np.where(inside, m / rho[None, :] * W(r), 0.0)
    v_x = v + c * (wgt[:, :, None] * vij).sum(1)
    g = G(r)[:, :, None] * d                                  # grad_i W
    vol = m / rho[None, :]                                    # neighbour volume m / rho_j
    w = (vol[:, :, None] * np.cross(vij, -g)).sum(1)          # sum_j V_j v_ij x grad_j W
    wm = np.linalg.norm(w, axis=1)
    eta = ((m / rho[None, :] * (wm[None, :] - wm[:, None]))[:, :, None] * g).sum(1)
    en = np.linalg.norm(eta, axis=1)
    N = np.where(en[:, None] > 1e-30, eta / np.maximum(en, 1e-300)[:, None], 0.0)
    f = eps * np.cross(N, w)
    if not bounds:
        return v_x + dt * f, w
    delta = 32 * np.finfo(np.float32).eps
    gn = np.linalg.norm(g, axis=-1)
    vn = np.linalg.norm(vij, axis=-1)
    d_w = delta * (vol * vn * gn).sum(1)                                # omega
    d_x = delta * c * (wgt * vn).sum(1)                                 # XSPH change
    mr = m / rho[None, :] * gn
    d_eta = delta * (mr * np.abs(wm[None, :] - wm[:, None])).sum(1) + (mr * (d_w[None, :] + d_w[:, None])).sum(1)
    d_N = 2.0 * d_eta / np.maximum(en, 1e-300)
    d_f = eps * (wm * np.minimum(d_N, 2.0) + d_w)
    return v_x + dt * f, w, d_x + dt * d_f, d_w


def clamped_lambda_numpy(pos, p):
    h, m = float(np.float32(p.h)), float(np.float32(p.mass))
    r0, eps = float(np.float32(p.rest_dens)), float(np.float32(p.epsilon))
    W, G = kernels(h)
    d, r = pairs(pos)
    rho = (m * W(r)).sum(1)
    g = G(r)[:, :, None] * d / r0
    sd = (g * g).sum(-1).sum(1) + (g.sum(1) ** 2).sum(-1)
    C = np.maximum(rho / r0 - 1.0, 0.0)
    return rho, -C / (sd + eps)


def test_xsph_vorticity_match_numpy():
    pos, vel, dens, p = state()
    dt = 0.0016
    v_np, w_np = xsph_vorticity_numpy(pos, vel, dens, p, dt)
    o = oracle.Oracle(p, pos.shape[0], threads=2)
    vo, wo = o.finalize_ext(pos, vel, dens, dt)
    assert_close(wo[:, :3], w_np, "vorticity omega")
    # the velocity change of both terms (the velocity itself would hide it);
    # the oracle stores v + dv in FP32, so dv carries one ulp of |v + dv|
    assert_close(vo[:, :3] - vel[:, :3], v_np - vel[:, :3].astype(np.float64), "XSPH + confinement velocity change",
                 atol=ulp32(vo[:, :3]))
    # each term on its own: XSPH alone, then confinement alone
    for c, e in ((0.01, 0.0), (0.0, 1e-4)):
        p1 = abi.FsphParams.from_buffer_copy(p)
        p1.xsph_c, p1.vort_eps = c, e
        v1, _ = xsph_vorticity_numpy(pos, vel, dens, p1, dt)
        o1 = oracle.Oracle(p1, pos.shape[0], threads=2)
        vo1, _ = o1.finalize_ext(pos, vel, dens, dt)
        assert_close(vo1[:, :3] - vel[:, :3], v1 - vel[:, :3].astype(np.float64), f"velocity change c={c} eps={e}",
                     atol=ulp32(vo1[:, :3]))


def test_clamped_lambda_matches_numpy():
    pos, _, _, p = state(seed=12)
    # squeeze the block so that part of it is over-dense (C > 0) and part,
    # the surface, under-dense (C clamped to 0)
    pos = pos.copy()
    pos[:, :3] = pos[:, :3].mean(0) + 0.93 * (pos[:, :3] - pos[:, :3].mean(0))
    p.clamp_constraint = 1
    rho_np, lam_np = clamped_lambda_numpy(pos, p)
    o = oracle.Oracle(p, pos.shape[0], threads=2)
    rho, lam = o.lambda_pass(pos)
    assert (lam_np == 0).any() and (lam_np < 0).any()
    assert_close(rho, rho_np, "density")
    assert_close(lam, lam_np, "clamped lambda")
    assert np.array_equal(lam == 0, lam_np == 0), "the clamp zeroes the same particles"
