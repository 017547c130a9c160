"""Seeded synthetic scenes: the replacement of the reference's scene loader.

The reference fills its particles through rxSPHConfig::SetLiquidBox ->
rxParticleSystemBase::AddBox (rx_sph_config.h:257-269, rx_ps.cpp:195-261): a
cubic lattice with a small uniform jitter drawn from ``srand(time(NULL))``.
Here the same kind of block is drawn from a counter-based generator
(SplitMix64 of (seed, stream, particle index)), so a scene is the same bytes
on every machine and in every process, and the CPU oracle and the GPU run
start from identical states.

Workloads (the configurations the fluid step is measured on):
  wcsph_dam_break      32^3 WCSPH dam break; h = 0.0457, m = 0.02, rho0 = 998.29,
                       k = 3, mu = 3.5 / rho0, dt = 1e-3, 200 steps
  pbf_dam_break        64^3 PBF dam break; eps = 100, 4 iterations, s_corr k=0.1 n=4
                       q=0.2, XSPH c = 0.01, vorticity 1e-4, dt = 0.0016
  pbf_double_dam_break 1,048,576 particles in two 64x64x128 blocks (the benchmark
                       workload); iterate to mean one-sided density error <= 0.1 %
  batched_scenes       256 independent PBF scenes, N_s log-uniform in [2048, 65536]

Geometry: every lattice has spacing h/2 (about 33 neighbours per particle),
the particle radius used by the walls is h/4 (half the spacing), and the
boxes are sized so the stated blocks fit at the stated h; the particle mass
is the one for which the h/2 lattice sums to rho0 (PBF configurations).
Box sides are the longest side divided by powers of two (or within a factor
sqrt(2) above one): the reference's CPU grid rounds every axis to a
power-of-two cell count (rx_nnsearch.h:174-217) and, when an axis rounds
down, leaves the far end of the box outside the grid, where its neighbour
query then misses neighbours.  With these ratios its grid covers the box and
its neighbour sets are the geometric ones.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import abi

H_DEFAULT = 0.0457
REST_DENS = 998.29

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea, Flood 2014), vectorised over uint64."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    """U[0,1) doubles, one per index, from (seed, stream, idx)."""
    with np.errstate(over="ignore"):
        base = splitmix64(np.array([(seed * 0x100000001B3 + stream) & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64))[0]
        x = splitmix64((idx.astype(np.uint64) * np.uint64(0xD1B54A32D192ED03)) ^ base)
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def poly6(r: np.ndarray, h: float) -> np.ndarray:
    aw = 315.0 / (64.0 * math.pi * h ** 9)
    q = h * h - r * r
    return np.where((r >= 0) & (r <= h), aw * q * q * q, 0.0)


def lattice_mass(h: float, spacing: float, rest_dens: float = REST_DENS) -> float:
    """Mass for which a cubic lattice of the given spacing has density rest_dens
    (the inverse of calRestDensity, rx_sph_pbd.cpp:1035-1049)."""
    n = int(math.ceil(h / spacing)) + 1
    ax = np.arange(-n, n + 1) * spacing
    x, y, z = np.meshgrid(ax, ax, ax, indexing="ij")
    s = poly6(np.sqrt(x * x + y * y + z * z), h).sum()
    return float(rest_dens / s)


def lattice_block(origin, dims, spacing: float, jitter: float, seed: int, stream: int) -> np.ndarray:
    """float32 (N, 4) positions of a jittered cubic lattice, x fastest
    (the loop order of AddBox, rx_ps.cpp:215-240), w = 0."""
    nx, ny, nz = (int(d) for d in dims)
    n = nx * ny * nz
    idx = np.arange(n, dtype=np.int64)
    i = idx % nx
    j = (idx // nx) % ny
    k = idx // (nx * ny)
    pos = np.zeros((n, 4), dtype=np.float64)
    for a, (o, c) in enumerate(zip(origin, (i, j, k))):
        u = uniform(seed, stream * 3 + a, idx)
        pos[:, a] = o + c * spacing + (2.0 * u - 1.0) * jitter
    return pos.astype(np.float32)


@dataclasses.dataclass
class Scene:
    name: str
    pos: np.ndarray          # (N, 4) float32
    vel: np.ndarray          # (N, 4) float32
    params: abi.FsphParams
    dt: float
    steps: int
    fixed_iters: int = 0     # > 0: run exactly this many PBF iterations per step
    boundary: np.ndarray | None = None   # (NB, 4) float32 static boundary particles

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def pbf_params(h: float, box_min, box_max, n: int, **kw) -> abi.FsphParams:
    p = abi.FsphParams()
    p.solver = abi.SOLVER_PBF
    p.max_particles = n
    p.h = h
    p.rest_dens = REST_DENS
    p.mass = lattice_mass(h, 0.5 * h)
    p.particle_radius = 0.25 * h
    for a in range(3):
        p.box_min[a] = box_min[a]
        p.box_max[a] = box_max[a]
    p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, -9.81, 0.0
    p.viscosity = 0.0
    p.gas_k = 3.0
    p.epsilon = 100.0
    p.eta = 1e-3
    p.min_iter = 2
    p.max_iter = 100
    p.error_mode = abi.ERR_ONE_SIDED
    p.use_ap = 1
    p.ap_k, p.ap_n, p.ap_q = 0.1, 4.0, 0.2
    p.xsph_c = 0.01
    p.vort_eps = 1e-4
    p.cell_skin = 0.05
    p.use_graph = 1
    p.warm_start = 0
    p.mlp_tcgen05 = 1
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _block_origin(box_min, h):
    s = 0.5 * h
    return [b + 0.5 * s + 0.01 * h for b in box_min]


def wcsph_dam_break(n_side: int = 32, h: float = H_DEFAULT, seed: int = 1) -> Scene:
    """32^3 WCSPH dam break.  The stated [0,1]x[0,0.6]x[0,0.4] box cannot hold a
    32^3 block at spacing h/2 (0.73 m per side), so the box is enlarged to
    [0,2]x[0,1]x[0,1].  mu = 3.5 / rho0: the reference multiplies an
    acceleration by mu (rx_sph_cpu.cpp:626-633), and mu = 3.5 is unstable at dt = 1e-3."""
    s = 0.5 * h
    scale = max(1.0, n_side / 32.0)
    box_min = [0.0, 0.0, 0.0]
    box_max = [2.0 * scale, 1.0 * scale, 1.0 * scale]
    pos = lattice_block(_block_origin(box_min, h), (n_side, n_side, n_side), s, 0.01 * h, seed, 0)
    p = pbf_params(h, box_min, box_max, pos.shape[0])
    p.solver = abi.SOLVER_WCSPH
    p.mass = 0.02
    p.rest_dens = REST_DENS
    p.gas_k = 3.0
    p.viscosity = 3.5 / REST_DENS
    p.xsph_c = 0.0
    p.vort_eps = 0.0
    return Scene("wcsph_dam_break", pos, np.zeros_like(pos), p, 1e-3, 200)


def pbf_dam_break(n_side: int = 64, h: float = H_DEFAULT, seed: int = 2) -> Scene:
    """64^3 PBF dam break with 4 fixed iterations.  The stated 1x1x0.5 box
    cannot hold a 64^3 block at spacing h/2 (1.46 m), so it is scaled by 3."""
    s = 0.5 * h
    ext = n_side * s
    box_min = [0.0, 0.0, 0.0]
    L = max(1.0, 2.05 * ext)
    box_max = [L, L, 0.5 * L]
    pos = lattice_block(_block_origin(box_min, h), (n_side, n_side, n_side), s, 0.01 * h, seed, 0)
    p = pbf_params(h, box_min, box_max, pos.shape[0])
    return Scene("pbf_dam_break", pos, np.zeros_like(pos), p, 0.0016, 500, fixed_iters=4)


def pbf_double_dam_break(block=(64, 64, 128), h: float = H_DEFAULT, seed: int = 3,
                         eta: float = 1e-3) -> Scene:
    """Two water columns at opposite ends of a long box collapsing toward each
    other; with the default 64x64x128 blocks, 1,048,576 particles.  The box is
    L x L/4 x L/2 with L = 4.1 block widths (blocks with by <= bx, bz <= 2 bx);
    columns taller than wide (bx < by <= 2 bx) get a box L/2 high."""
    s = 0.5 * h
    bx, by, bz = block
    if by > 2 * bx or bz > 2 * bx:
        raise ValueError("block must satisfy by <= 2 bx and bz <= 2 bx")
    L = 4.1 * bx * s
    box_min = [0.0, 0.0, 0.0]
    box_max = [L, (0.25 if by <= bx else 0.5) * L, 0.5 * L]
    o = _block_origin(box_min, h)
    a = lattice_block(o, block, s, 0.01 * h, seed, 0)
    o2 = [box_max[0] - o[0] - (bx - 1) * s, o[1], o[2]]
    b = lattice_block(o2, block, s, 0.01 * h, seed, 1)
    pos = np.concatenate([a, b])
    p = pbf_params(h, box_min, box_max, pos.shape[0], eta=eta)
    return Scene("pbf_double_dam_break", pos, np.zeros_like(pos), p, 0.0016, 500)


def batched_scenes(count: int = 256, seed: int = 4, n_lo: int = 2048, n_hi: int = 65536,
                   h: float = H_DEFAULT) -> list[Scene]:
    """Independent PBF scenes: N_s log-uniform in [n_lo, n_hi], box sides
    uniform in [0.3, 1.0] (the box's proportions), fill fraction uniform in
    [0.2, 0.5].  As in the other workloads h and the constants stay fixed
    (spacing h/2, ~33 neighbours) and the box is scaled so that the N_s-
    particle block fills the stated fraction of it: with the stated 0.3-1.0
    sides themselves h would have to shrink per scene, and at the fixed
    dt = 0.0016 the reference's dt^2-scaled s_corr term then dominates lambda
    in the small-h scenes and the step diverges (seen on the CPU oracle)."""
    idx = np.arange(count, dtype=np.int64)
    un = uniform(seed, 100, idx)
    ub = [uniform(seed, 101 + a, idx) for a in range(3)]
    uf = uniform(seed, 104, idx)
    sp = 0.5 * h
    out = []
    for s_i in range(count):
        n_target = int(round(math.exp(math.log(n_lo) + un[s_i] * (math.log(n_hi) - math.log(n_lo)))))
        shape = [0.3 + 0.7 * ub[a][s_i] for a in range(3)]
        fill = 0.2 + 0.3 * uf[s_i]
        scale = (n_target * sp ** 3 / (fill * shape[0] * shape[1] * shape[2])) ** (1.0 / 3.0)
        L = [scale * shape[a] for a in range(3)]
        ext = [L[a] * fill ** (1.0 / 3.0) for a in range(3)]
        dims = [max(2, int(round(e / sp))) for e in ext]
        box_max = [max(L[a], dims[a] * sp + 0.05 * h) for a in range(3)]
        pos = lattice_block(_block_origin([0, 0, 0], h), dims, sp, 0.01 * h, seed + 1000 + s_i, 0)
        p = pbf_params(h, [0, 0, 0], box_max, pos.shape[0])
        out.append(Scene(f"batched_{s_i}", pos, np.zeros_like(pos), p, 0.0016, 500, fixed_iters=4))
    return out


def box_surface(lo, side: float, spacing: float, layers: int = 1) -> np.ndarray:
    """Particles on the surface of the axis-aligned cube [lo, lo + side]^3: the
    lattice points of an m^3 grid (m = side / spacing, rounded) that lie on
    the cube's faces, each once -- the role of rxSolid::GenerateParticlesOnSurf
    for a box (rx_sph_pbd.cpp:180, spacing 1.2 r there).  layers > 1 keeps
    every lattice point within layers - 1 spacings of a face (a solid shell)."""
    m = max(1, int(round(side / spacing)))
    s = side / m
    g = np.arange(m + 1)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    depth = np.minimum.reduce([x, m - x, y, m - y, z, m - z])
    on = depth < max(1, int(layers))
    pts = np.stack([x[on], y[on], z[on]], axis=1).astype(np.float64) * s + np.asarray(lo, np.float64)
    out = np.zeros((pts.shape[0], 4), np.float32)
    out[:, :3] = pts
    return out


def pbf_obstacle_drop(n_side: int = 256, h: float = H_DEFAULT, seed: int = 5) -> Scene:
    """An n_side^3 jittered block (spacing h/2) dropped onto a static box
    obstacle made of boundary particles (the 16,777,216-particle configuration
    at n_side = 256).  The stated 2 x 2 x 2 box and 0.3 obstacle keep their
    proportions, scaled so the block fits at the stated h: box L^3 with L =
    2.6 block sides, obstacle side 0.15 L at the centre, block centred in x and
    z one h above it (so the impact starts within a few steps).  Obstacle
    particles at spacing 1.2 r (r = h / 4), the reference's surface spacing
    for solids, in a shell of 10 layers (3 h thick): 1.48M boundary particles
    at n_side = 256, the stated ~1.5M.  Only the outer layers meet the fluid
    (within h); the deeper ones give the outer layers the boundary volume
    psi_b of a solid rather than of a sheet."""
    s = 0.5 * h
    B = n_side * s
    L = 2.6 * B
    ob_side = 0.15 * L
    ob_lo = [0.5 * (L - ob_side)] * 3
    bnd = box_surface(ob_lo, ob_side, 1.2 * 0.25 * h, layers=10)
    o = [0.5 * (L - B) + 0.5 * s, ob_lo[1] + ob_side + h + 0.5 * s, 0.5 * (L - B) + 0.5 * s]
    pos = lattice_block(o, (n_side, n_side, n_side), s, 0.01 * h, seed, 0)
    p = pbf_params(h, [0, 0, 0], [L, L, L], pos.shape[0])
    return Scene("pbf_obstacle_drop", pos, np.zeros_like(pos), p, 0.0016, 100, boundary=bnd)
