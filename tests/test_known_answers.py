"""Known-answer tests of the oracle that the reference does not ship (it has
no tests): kernel normalisation, hand-computed lambda, lattice neighbour
count, pair-force momentum balance, FP32 vs FP64 drift.  CPU only."""
import math

import numpy as np

import oracle
from fltk_sph_ice_gb300 import abi, scenes


def test_poly6_normalised():
    L = oracle.orc_lib()
    h = 0.0457
    r = np.linspace(0.0, h, 20001)
    w = np.array([L.fsph_orc_kernel(0, float(x), h) for x in r])
    integral = np.trapezoid(4.0 * math.pi * r * r * w, r)
    assert abs(integral - 1.0) < 1e-6


def test_spiky_gradient_is_derivative_of_spiky():
    L = oracle.orc_lib()
    h = 0.0457
    a = 15.0 / (math.pi * h ** 6)  # spiky W = a (h - r)^3
    for r in np.linspace(0.05 * h, 0.95 * h, 7):
        dwdr = -3.0 * a * (h - r) ** 2
        assert abs(L.fsph_orc_kernel(1, float(r), h) * r - dwdr) <= 1e-9 * abs(dwdr)


def test_lattice_neighbour_count_is_33():
    """An interior particle of a perfect h/2 lattice has 33 neighbours (self included).
    The spacing is a hair below h/2 so that the six axis neighbours at exactly h
    are not decided by the rounding of float positions."""
    h = 0.0457
    s = 0.4999 * h
    g = np.arange(9) * s + 0.2
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.zeros((x.size, 4), np.float32)
    pos[:, 0], pos[:, 1], pos[:, 2] = x.ravel(), y.ravel(), z.ravel()
    p = scenes.pbf_params(h, [0, 0, 0], [1, 1, 1], pos.shape[0])
    o = oracle.Oracle(p, pos.shape[0])
    off, idx = o.neighbors(pos)
    centre = 4 * 81 + 4 * 9 + 4
    assert off[centre + 1] - off[centre] == 33


def test_two_particle_lambda_by_hand():
    h = 0.0457
    r = 0.5 * h
    p = scenes.pbf_params(h, [0, 0, 0], [1, 1, 1], 2)
    pos = np.array([[0.5, 0.5, 0.5, 0], [0.5 + r, 0.5, 0.5, 0]], np.float32)
    o = oracle.Oracle(p, 2, "double")
    d, lam = o.lambda_pass(pos)
    aw = 315.0 / (64.0 * math.pi * h ** 9)
    rr = float(pos[1, 0]) - float(pos[0, 0])
    rho = p.mass * (aw * h ** 6 + aw * (h * h - rr * rr) ** 3)
    g = 45.0 / (math.pi * h ** 6) * (h - rr) ** 2 / p.rest_dens
    C = rho / p.rest_dens - 1.0
    lam_hand = -C / (2.0 * g * g + p.epsilon)
    assert abs(d[0] - rho) <= 1e-6 * rho
    assert abs(lam[0] - lam_hand) <= 1e-6 * abs(lam_hand)


def test_wcsph_pressure_forces_balance_momentum():
    sc = scenes.wcsph_dam_break(n_side=8)
    p = sc.params
    p.viscosity = 0.0
    p.gravity[1] = 0.0
    x = sc.pos.copy()
    x[:, :3] = x[:, :3].mean(0) + (x[:, :3] - x[:, :3].mean(0)) * 0.95
    o = oracle.Oracle(p, sc.n, "double")
    d, pr, a = o.sph_forces(x, np.zeros_like(x))
    total = np.abs(a[:, :3].sum(0)).max()
    assert total <= 1e-6 * np.abs(a[:, :3]).sum()  # float32 outputs


def test_fp32_vs_fp64_oracle_drift():
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    p = sc.params
    p.eta, p.max_iter = 0.0, 4
    o32 = oracle.Oracle(p, sc.n, "float")
    o64 = oracle.Oracle(p, sc.n, "double")
    o32.set(sc.pos, sc.vel)
    o64.set(sc.pos, sc.vel)
    for _ in range(5):
        o32.pbf_step(sc.dt)
        o64.pbf_step(sc.dt)
    x32, x64 = o32.get("pos"), o64.get("pos")
    drift = np.abs(x32.astype(np.float64) - x64).max() / np.abs(x64).max()
    assert drift < 1e-5, drift


def test_rest_density_of_reference_defaults():
    L = oracle.orc_lib()
    # kp = 20, m = 0.02, rho = 998.29: h = 0.04573, r = 0.01358, rho0 = 961.2326 (rx_sph_pbd.cpp:110-135)
    h = (3.0 * 20 * 0.02 / (4.0 * math.pi * 998.29)) ** (1.0 / 3.0)
    r = (math.pi / (6.0 * 20)) ** (1.0 / 3.0) * h
    rho0 = L.fsph_orc_lattice_density(h, 0.02, 2.0 * np.float32(r))
    assert abs(rho0 - 961.2326) < 2e-3


def test_lattice_mass_inverts_rest_density():
    L = oracle.orc_lib()
    h = 0.0457
    m = scenes.lattice_mass(h, 0.5 * h)
    rho = L.fsph_orc_lattice_density(h, m, 0.5 * h)
    assert abs(rho - scenes.REST_DENS) <= 1e-5 * scenes.REST_DENS
    assert abs(m - 0.011795) < 1e-5


def test_scene_generation_is_deterministic():
    a = scenes.pbf_double_dam_break(block=(8, 8, 16))
    b = scenes.pbf_double_dam_break(block=(8, 8, 16))
    c = scenes.pbf_double_dam_break(block=(8, 8, 16), seed=99)
    assert np.array_equal(a.pos, b.pos)
    assert not np.array_equal(a.pos, c.pos)
    full = scenes.pbf_double_dam_break()
    assert full.n == 1 << 20
    assert (full.pos[:, :3] >= np.array(full.params.box_min) + full.params.particle_radius - 0.011 * full.params.h).all()
    for sc in (full, scenes.pbf_dam_break(), scenes.wcsph_dam_break()):
        lmax = max(sc.params.box_max[a] - sc.params.box_min[a] for a in range(3))
        for a in range(3):
            ratio = math.log2(lmax / (sc.params.box_max[a] - sc.params.box_min[a]))
            assert ratio - math.floor(ratio) < 0.5 or abs(ratio - round(ratio)) < 1e-9, (sc.name, a)


def test_batched_scene_statistics():
    sl = scenes.batched_scenes(count=64)
    ns = np.array([s.n for s in sl])
    assert ns.min() >= 1500 and ns.max() <= 80000
    assert all(s.params.solver == abi.SOLVER_PBF for s in sl)
