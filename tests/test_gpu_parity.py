"""GPU parity: the sm_103a kernels, called through the C ABI, against the
reference's own CPU code (golden vectors) and the CPU oracle.

Bars: neighbour sets bit-exact; density / lambda / delta-p / force and
positions within 1e-5 in max|a-b| / max|b| (FP32 against the reference's
float-storage, double-geometry arithmetic)."""
import numpy as np
import pytest

import oracle
from conftest import assert_close, assert_rel, assert_same_sets, golden, params_from_golden, ulp32
from fltk_sph_ice_gb300 import FsphError, abi, rxPBDSPH, rxSPH, scenes

pytestmark = pytest.mark.gpu


def test_neighbour_sets_match_reference(gpu):
    g = golden("pbf_small")
    ps = rxPBDSPH(params_from_golden(g))
    ps.Set(g["pos"])
    off, idx = ps.GetNeights()
    assert_same_sets(off, idx, g["nb_off"], g["nb_idx"])


def test_neighbour_sets_after_dynamics(gpu):
    """Sets on a splashing state (oracle-evolved), compared on identical positions."""
    sc = scenes.pbf_double_dam_break(block=(10, 10, 20))
    p = sc.params
    p.max_iter = 6
    o = oracle.Oracle(p, sc.n, threads=4)
    o.set(sc.pos, sc.vel)
    for _ in range(40):
        o.pbf_step(sc.dt)
    x = o.get("pos")
    ps = rxPBDSPH(p)
    ps.Set(x)
    off, idx = ps.GetNeights()
    off_o, idx_o = o.neighbors(x)
    assert_same_sets(off, idx, off_o, idx_o)
    assert np.diff(off).max() > np.diff(off).min()


def test_lambda_pass_matches_reference(gpu):
    g = golden("pbf_small")
    ps = rxPBDSPH(params_from_golden(g))
    d, lam = ps.EvalScalingFactor(g["pos"])
    assert_rel(d, g["dens"], 1e-5, "density")
    assert_rel(lam, g["lam"], 1e-5, "lambda")


def test_correction_pass_matches_reference(gpu):
    g = golden("pbf_small")
    ps = rxPBDSPH(params_from_golden(g))
    dp = ps.EvalPositionCorrection(g["pos"], g["lam"], float(g["dt"]))
    assert_rel(dp, g["dp"], 1e-5, "delta p")


@pytest.mark.parametrize("use_graph", [0, 1])
def test_pbf_steps_match_reference(gpu, use_graph):
    g = golden("pbf_small")
    p = params_from_golden(g)
    p.use_graph = use_graph
    ps = rxPBDSPH(p)
    ps.Set(g["pos"], g["vel"])
    for k in range(3):
        ps.Update(float(g["dt"]))
        assert ps.last_stats.iterations == g["step_iters"][k] == 4
        assert abs(ps.last_stats.density_error_two_sided - g["step_eta"][k]) <= 1e-4 * g["step_eta"][k]
        assert_rel(ps.GetArrayVBO(abi.RX_POSITION), g["step_pos"][k], 1e-5, f"positions after step {k + 1}")


@pytest.mark.parametrize("variant", ["one_sided_tol", "clamped_tol", "xsph_vort", "viscous_prepass"])
def test_pbf_variants_match_oracle(gpu, variant):
    sc = scenes.pbf_double_dam_break(block=(10, 10, 20))
    p = sc.params
    p.xsph_c, p.vort_eps = 0.0, 0.0
    p.max_iter, p.min_iter = 30, 2
    if variant == "one_sided_tol":
        p.eta = 2e-3
    elif variant == "clamped_tol":
        p.clamp_constraint, p.eta = 1, 1e-3
    elif variant == "xsph_vort":
        p.xsph_c, p.vort_eps, p.max_iter, p.eta = 0.01, 1e-4, 4, 0.0
    elif variant == "viscous_prepass":
        p.viscosity, p.max_iter, p.eta = 0.05, 4, 0.0
    vel = np.zeros_like(sc.pos)
    vel[:, 0] = 0.2
    o = oracle.Oracle(p, sc.n, threads=4)
    o.set(sc.pos, vel)
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, vel)
    xg0, xo0 = sc.pos[:, :3].astype(np.float64), sc.pos[:, :3].astype(np.float64)
    for k in range(2):
        it, errs = o.pbf_step(sc.dt)
        ps.Update(sc.dt)
        assert ps.last_stats.iterations == it, (k, ps.last_stats.iterations, it)
        xg, xo = ps.GetArrayVBO(abi.RX_POSITION)[:, :3], o.get("pos")[:, :3]
        assert_rel(xg, xo, 1e-5, f"{variant} positions step {k + 1}")
        # the step's position change, up to one ulp of each stored position
        store = ulp32(xo) + ulp32(xo0)
        assert_close(xg - xg0, xo - xo0, f"{variant} position change step {k + 1}",
                     atol=store + np.abs(xg0 - xo0))
        # v = (x* - x) / dt (then XSPH, which averages over neighbours with
        # weights summing to c (1 + ...) < 0.05): its error is the position
        # differences of both ends over dt, taken at their largest
        dv = 1.05 * (np.abs(xg - xo) + np.abs(xg0 - xo0) + store).max() / sc.dt
        assert_close(ps.GetArrayVBO(abi.RX_VELOCITY)[:, :3], o.get("vel")[:, :3], f"{variant} velocities step {k + 1}",
                     atol=dv)
        assert_rel(ps.GetArrayVBO(abi.RX_DENSITY), o.get("dens"), 1e-5, f"{variant} density step {k + 1}")
        xg0, xo0 = xg.astype(np.float64), xo.astype(np.float64)
    if variant == "xsph_vort":
        # omega = sum_j (m / rho_j)(v_j - v_i) x grad_j W: the velocity error
        # above times 2 sum_j (m / rho_j) |grad W_ij| (at most 2 dv per pair),
        # plus the FP32 rounding of the terms (32 eps x the sum of their sizes)
        off, idx = o.neighbors(o.get("pos"))
        rows = np.repeat(np.arange(sc.n), np.diff(off))
        x, v = o.get("pos")[:, :3].astype(np.float64), o.get("vel")[:, :3].astype(np.float64)
        d = x[rows] - x[idx]
        r = np.sqrt((d * d).sum(1))
        h = float(np.float32(p.h))
        rho = o.get("dens").astype(np.float64)
        gw = np.where((r > 0) & (r <= h), 45.0 / (np.pi * h ** 6) * (h - r) ** 2, 0.0) * float(p.mass) / rho[idx]
        sg = np.bincount(rows, weights=gw, minlength=sc.n)
        sv = np.bincount(rows, weights=gw * np.linalg.norm(v[idx] - v[rows], axis=1), minlength=sc.n)
        bound = 2.0 * dv * sg + 32 * np.finfo(np.float32).eps * sv
        assert_close(ps.GetArrayVBO(abi.RX_VORTICITY)[:, :3], o.get("vort")[:, :3], "vorticity",
                     atol=bound[:, None])


def test_xsph_vorticity_pass_matches_numpy(gpu):
    """The end-of-step XSPH + vorticity-confinement passes alone, against the
    brute-force numpy restatement that pins the oracle
    (tests/test_extensions_oracle.py), on a swirling jittered block:
    norm-wise 1e-5 and element-wise 1e-4 above 1 % of the largest entry,
    each plus the first-order FP32 rounding bound of the particle's pair
    terms (and one ulp of the stored velocity for the velocity change)."""
    from test_extensions_oracle import state, xsph_vorticity_numpy
    pos, vel, dens, p = state(seed=21, dims=(14, 12, 12))
    dt = 0.0016
    v_np, w_np, d_v, d_w = xsph_vorticity_numpy(pos, vel, dens, p, dt, bounds=True)
    ps = rxPBDSPH(p)
    vo, wo = ps.EvalXsphVorticity(pos, vel, dens, dt)
    ps.close()
    assert_close(wo[:, :3], w_np, "omega", atol=d_w[:, None])
    assert_close(vo[:, :3] - vel[:, :3], v_np - vel[:, :3].astype(np.float64), "velocity change",
                 atol=d_v[:, None] + ulp32(vo[:, :3]))


def test_wcsph_matches_reference(gpu):
    g = golden("sph_small")
    p = params_from_golden(g)
    ws = rxSPH(p)
    d, pr, a = ws.EvalForces(g["pos"], g["vel"])
    assert_rel(d, g["dens"], 1e-5, "density")
    assert_rel(pr, g["pres"], 1e-5, "pressure")
    assert_rel(a, g["frc"], 1e-5, "acceleration")
    ws.Set(g["pos"], g["vel"])
    for k in range(5):
        ws.Update(float(g["dt"]))
        assert_rel(ws.GetArrayVBO(abi.RX_POSITION), g["step_pos"][k], 1e-5, f"positions after step {k + 1}")


def test_fp64_error_report(gpu):
    """Error of every FP32 result against the FP64 oracle on the same inputs."""
    g = golden("pbf_small")
    p = params_from_golden(g)
    n = g["pos"].shape[0]
    o64 = oracle.Oracle(p, n, "double")
    d64, l64 = o64.lambda_pass(g["pos"])
    dp64 = o64.correction_pass(g["pos"], l64, float(g["dt"]))
    ps = rxPBDSPH(p)
    d, lam = ps.EvalScalingFactor(g["pos"])
    dp = ps.EvalPositionCorrection(g["pos"], l64, float(g["dt"]))
    errs = {"density": (d, d64), "lambda": (lam, l64), "delta_p": (dp, dp64)}
    report = {k: float(np.abs(np.asarray(a, np.float64) - b).max() / np.abs(b).max()) for k, (a, b) in errs.items()}
    print("FP32 vs FP64 oracle:", report)
    for k, e in report.items():
        assert e < 1e-5, (k, e)


def test_neighbour_lists_match_cell_walk(gpu):
    """Lists visit the in-range candidates of the 27-cell walk in the walk's
    order: bit-identical passes at a build, equal steps within the parity bar."""
    sc = scenes.pbf_double_dam_break(block=(12, 12, 24))
    out = {}
    for wc in (0, 1):
        p = abi.FsphParams.from_buffer_copy(sc.params)
        p.walk_cells = wc
        ps = rxPBDSPH(p)
        d, lam = ps.EvalScalingFactor(sc.pos)
        ps.Set(sc.pos, sc.vel)
        its = []
        for _ in range(3):
            ps.Update(sc.dt)
            its.append(ps.last_stats.iterations)
        out[wc] = (d, lam, ps.GetArrayVBO(abi.RX_POSITION), its, ps.last_stats.grid_builds)
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    # the two paths visit neighbours in different orders once particles leave
    # their build cells, so whole steps agree to the parity bar, not bitwise
    assert_rel(out[0][2], out[1][2], 1e-5, "positions after 3 steps")
    assert out[0][3] == out[1][3]


def test_graph_and_eager_bit_identical(gpu):
    sc = scenes.pbf_double_dam_break(block=(12, 12, 24))
    out = []
    for ug in (0, 1):
        p = abi.FsphParams.from_buffer_copy(sc.params)
        p.use_graph = ug
        ps = rxPBDSPH(p)
        ps.Set(sc.pos, sc.vel)
        for _ in range(5):
            ps.Update(sc.dt)
        out.append((ps.GetArrayVBO(abi.RX_POSITION), ps.last_stats.iterations))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]


def test_edge_cases(gpu):
    sc = scenes.pbf_double_dam_break(block=(8, 8, 16))
    p = sc.params
    ps = rxPBDSPH(p)
    with pytest.raises(FsphError) as e:
        ps.Update(sc.dt)  # no particles: the reference's Update returns false
    assert e.value.status == abi.INVALID_ARG
    with pytest.raises(FsphError):
        ps.Set(np.zeros((sc.n + 1, 4), np.float32))  # beyond max_particles
    bad = sc.pos.copy()
    bad[3, 1] = np.nan
    with pytest.raises(FsphError) as e:
        ps.Set(bad)
    assert e.value.status == abi.NAN_DETECTED
    # a single particle falls and rests on the floor at the particle radius
    one = np.array([[0.3, 0.2, 0.3, 0.0]], np.float32)
    ps.Set(one)
    for _ in range(200):
        ps.Update(sc.dt)
    y = ps.GetArrayVBO(abi.RX_POSITION)[0, 1]
    assert abs(y - (p.box_min[1] + p.particle_radius)) < 1e-6
    # particles placed outside the box are projected onto the walls
    out = sc.pos.copy()
    out[:10, 0] = -1.0
    ps.Set(out)
    ps.Update(sc.dt)
    x = ps.GetArrayVBO(abi.RX_POSITION)
    assert (x[:, 0] >= p.box_min[0] + p.particle_radius - 1e-6).all()
