"""CPU oracle of the fluid step -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, by ``__graft_entry__.smoke()`` (as the checker) and by the
CPU-baseline leg of ``bench.py``.  The product package never imports it.

Two libraries:
  * ``_build/libfsph_oracle.so``  -- this project's restatement of the
    reference CPU path (fsph_oracle.cpp), in float (reference arithmetic) or
    double (FP64 oracle);
  * ``_ref/libfsph_ref.so``       -- the reference's OWN CPU fluid functions,
    compiled by ref_harness/extract.py, which pins the restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
ORC_LIB = os.path.join(BUILD, "libfsph_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfsph_ref.so")

_orc = None
_ref = None


def build_oracle() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "fsph_oracle.cpp")
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-ffp-contract=off",
           src, "-o", ORC_LIB]
    if (not os.path.isfile(ORC_LIB)) or os.path.getmtime(ORC_LIB) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "..", "include", "fsph.h"))):
        subprocess.run(cmd, check=True)
    return ORC_LIB


def build_reference() -> str | None:
    from .ref_harness.extract import build_ref
    return build_ref()


def _vp(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f4(a, n: int) -> np.ndarray:
    """a contiguous float32 (n, 4) array (the C side reads 4 n floats)"""
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.shape != (n, 4):
        raise ValueError(f"expected a float4 array of shape ({n}, 4), got {a.shape}")
    return a


def orc_lib() -> ctypes.CDLL:
    global _orc
    if _orc is None:
        build_oracle()
        L = ctypes.CDLL(ORC_LIB)
        vp, ci, cf, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
        L.fsph_orc_create.restype = vp
        L.fsph_orc_create.argtypes = [vp, ci, ci]
        L.fsph_orc_destroy.argtypes = [vp]
        L.fsph_orc_set.argtypes = [vp, vp, vp]
        L.fsph_orc_get.argtypes = [vp, ci, vp]
        L.fsph_orc_set_boundary.argtypes = [vp, vp, ci]
        L.fsph_orc_get_boundary.argtypes = [vp, ci, vp]
        L.fsph_orc_pbf_step.argtypes = [vp, cf, ci, vp]
        L.fsph_orc_pbf_step.restype = ci
        L.fsph_orc_sph_step.argtypes = [vp, cf]
        L.fsph_orc_finalize_ext.argtypes = [vp, vp, vp, vp, cf, vp, vp]
        L.fsph_orc_set_obstacles.argtypes = [vp, vp, ci]
        L.fsph_orc_project.argtypes = [vp, vp, ci, vp]
        L.fsph_orc_density_grid.argtypes = [vp, vp, vp, vp, vp]
        L.fsph_orc_set_polygons.argtypes = [vp, vp, ci, vp, ci]
        L.fsph_orc_polygon_collide.argtypes = [vp, vp, vp, vp, ci, cf]
        L.fsph_orc_neighbors.argtypes = [vp, vp, vp, vp, ctypes.c_longlong]
        L.fsph_orc_neighbors.restype = ctypes.c_longlong
        L.fsph_orc_pbf_lambda.argtypes = [vp, vp, vp, vp]
        L.fsph_orc_pbf_correction.argtypes = [vp, vp, vp, cf, vp]
        L.fsph_orc_sph_forces.argtypes = [vp, vp, vp, vp, vp, vp]
        L.fsph_orc_pbf_predict.argtypes = [vp, cf, vp, vp, vp, vp]
        L.fsph_orc_kernel.restype = cd
        L.fsph_orc_kernel.argtypes = [ci, cd, cd]
        L.fsph_orc_lattice_density.restype = cd
        L.fsph_orc_lattice_density.argtypes = [cd, cd, cd]
        L.fsph_orc_wall.argtypes = [vp, vp, vp]
        L.fsph_orc_threads.argtypes = [ci]
        _orc = L
    return _orc


class Oracle:
    """One CPU oracle instance (precision 'float' = reference arithmetic, 'double' = FP64)."""

    def __init__(self, params, n: int, precision: str = "float", threads: int = 0):
        self.L = orc_lib()
        self.n = int(n)
        self.params = params
        if threads:
            self.L.fsph_orc_threads(threads)
        self.h = self.L.fsph_orc_create(ctypes.byref(params), 1 if precision == "double" else 0, self.n)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fsph_orc_destroy(self.h)
            self.h = None

    def set(self, pos4, vel4=None):
        pos4 = _f4(pos4, self.n)
        vel4 = None if vel4 is None else np.ascontiguousarray(vel4, dtype=np.float32)
        self.L.fsph_orc_set(self.h, _vp(pos4), _vp(vel4))

    def get(self, which: str) -> np.ndarray:
        code = {"pos": 0, "vel": 1, "dens": 2, "lambda": 3, "dp": 4, "ppos": 5, "force": 6,
                "pres": 7, "vort": 8}[which]
        vec = which in ("pos", "vel", "dp", "ppos", "force", "vort")
        out = np.zeros((self.n, 4) if vec else (self.n,), dtype=np.float32)
        self.L.fsph_orc_get(self.h, code, _vp(out))
        return out

    def set_boundary(self, bpos4):
        """Static boundary particles (float4 positions); computes psi_b."""
        b = np.ascontiguousarray(bpos4, dtype=np.float32).reshape(-1, 4)
        self.nb = b.shape[0]
        self.L.fsph_orc_set_boundary(self.h, _vp(b), self.nb)

    def get_boundary(self, which: str) -> np.ndarray:
        out = np.zeros(getattr(self, "nb", 0), dtype=np.float32)
        self.L.fsph_orc_get_boundary(self.h, {"vol": 0, "lambda": 1}[which], _vp(out))
        return out

    def pbf_step(self, dt: float, fixed_iters: int = 0):
        errs = np.zeros(3, dtype=np.float64)
        it = self.L.fsph_orc_pbf_step(self.h, dt, fixed_iters, _vp(errs))
        return it, errs

    def sph_step(self, dt: float):
        self.L.fsph_orc_sph_step(self.h, dt)

    def set_obstacles(self, boxes=(), spheres=()):
        """Analytic obstacles: boxes as (cen, ext, ang_degrees), spheres as (cen, rad)."""
        rec = [[0.0, *c, *e, *a, 0.0] for c, e, a in boxes] + [[1.0, *c, 0, 0, 0, 0, 0, 0, r] for c, r in spheres]
        arr = np.ascontiguousarray(rec, dtype=np.float64).reshape(-1, 11)
        self.L.fsph_orc_set_obstacles(self.h, _vp(arr), arr.shape[0])

    def density_grid(self, n, minp, d):
        """The density field of the current positions on an n[0] x n[1] x n[2]
        lattice from minp with spacing d (CalImplicitField); (n[2], n[1], n[0])."""
        nn = np.ascontiguousarray(n, dtype=np.int32)
        out = np.zeros(int(np.prod(nn)), np.float32)
        self.L.fsph_orc_density_grid(self.h, _vp(nn), _vp(np.ascontiguousarray(minp, np.float64)),
                                     _vp(np.ascontiguousarray(d, np.float64)), _vp(out))
        return out.reshape(nn[2], nn[1], nn[0])

    def set_polygons(self, vrts, tris):
        """Triangle-mesh obstacles (vertices stored as floats, as the product does)."""
        v = np.ascontiguousarray(vrts, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
        self.L.fsph_orc_set_polygons(self.h, _vp(v), v.shape[0], _vp(t), t.shape[0])

    def polygon_collide(self, x0, x1, v, dt):
        a = np.ascontiguousarray(x0, np.float32)
        b = np.array(x1, np.float32, copy=True)
        c = np.array(v, np.float32, copy=True)
        self.L.fsph_orc_polygon_collide(self.h, _vp(a), _vp(b), _vp(c), a.shape[0], dt)
        return b, c

    def project(self, pos4):
        """The solid projection (obstacles, then the box walls) of the given points."""
        pos4 = _f4(pos4, len(pos4))
        out = np.zeros_like(pos4)
        self.L.fsph_orc_project(self.h, _vp(pos4), pos4.shape[0], _vp(out))
        return out

    def finalize_ext(self, pos4, vel4, dens, dt: float):
        """XSPH + vorticity confinement alone on the given state: (velocity after both, omega)."""
        pos4 = _f4(pos4, self.n)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        dens = np.ascontiguousarray(dens, dtype=np.float32)
        vo = np.zeros((self.n, 4), np.float32)
        om = np.zeros((self.n, 4), np.float32)
        self.L.fsph_orc_finalize_ext(self.h, _vp(pos4), _vp(vel4), _vp(dens), dt, _vp(vo), _vp(om))
        return vo, om

    def neighbors(self, pos4):
        pos4 = _f4(pos4, self.n)
        off = np.zeros(self.n + 1, dtype=np.int32)
        cap = self.n * 80
        idx = np.zeros(cap, dtype=np.int32)
        t = self.L.fsph_orc_neighbors(self.h, _vp(pos4), _vp(off), _vp(idx), cap)
        if t > cap:
            idx = np.zeros(t, dtype=np.int32)
            self.L.fsph_orc_neighbors(self.h, _vp(pos4), _vp(off), _vp(idx), t)
        return off, idx[:t]

    def lambda_pass(self, pos4):
        pos4 = _f4(pos4, self.n)
        d = np.zeros(self.n, np.float32)
        l = np.zeros(self.n, np.float32)
        self.L.fsph_orc_pbf_lambda(self.h, _vp(pos4), _vp(d), _vp(l))
        return d, l

    def correction_pass(self, pos4, lam, dt):
        pos4 = _f4(pos4, self.n)
        lam = np.ascontiguousarray(lam, dtype=np.float32)
        dp = np.zeros((self.n, 4), np.float32)
        self.L.fsph_orc_pbf_correction(self.h, _vp(pos4), _vp(lam), dt, _vp(dp))
        return dp

    def sph_forces(self, pos4, vel4):
        pos4 = _f4(pos4, self.n)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        d = np.zeros(self.n, np.float32)
        p = np.zeros(self.n, np.float32)
        a = np.zeros((self.n, 4), np.float32)
        self.L.fsph_orc_sph_forces(self.h, _vp(pos4), _vp(vel4), _vp(d), _vp(p), _vp(a))
        return d, p, a

    def pbf_predict(self, dt):
        d = np.zeros(self.n, np.float32)
        f = np.zeros((self.n, 4), np.float32)
        pp = np.zeros((self.n, 4), np.float32)
        pv = np.zeros((self.n, 4), np.float32)
        self.L.fsph_orc_pbf_predict(self.h, dt, _vp(d), _vp(f), _vp(pp), _vp(pv))
        return d, f, pp, pv


# --------------------------------------------------------------------------
# the reference's own CPU code (oracle/_ref)
# --------------------------------------------------------------------------
class RefEnv(ctypes.Structure):
    _fields_ = [("max_particles", ctypes.c_int), ("boundary_cen", ctypes.c_double * 3),
                ("boundary_ext", ctypes.c_double * 3), ("dens", ctypes.c_float), ("mass", ctypes.c_float),
                ("kernel_particles", ctypes.c_float), ("viscosity", ctypes.c_float), ("gas_k", ctypes.c_float),
                ("epsilon", ctypes.c_float), ("eta", ctypes.c_float), ("min_iter", ctypes.c_int),
                ("max_iter", ctypes.c_int), ("use_ap", ctypes.c_int), ("ap_k", ctypes.c_float),
                ("ap_n", ctypes.c_float), ("ap_q", ctypes.c_float), ("h", ctypes.c_float),
                ("particle_radius", ctypes.c_float), ("rest_dens", ctypes.c_float), ("gravity_y", ctypes.c_float)]


def ref_lib() -> ctypes.CDLL | None:
    """The reference-code library, built on demand; None when unavailable."""
    global _ref
    if _ref is None:
        if not os.path.isfile(REF_LIB):
            try:
                if build_reference() is None:
                    return None
            except Exception:
                return None
        L = ctypes.CDLL(REF_LIB)
        vp, ci, cf, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
        for pre in ("pbf", "sph"):
            getattr(L, f"fsph_ref_{pre}_create").restype = vp
            getattr(L, f"fsph_ref_{pre}_create").argtypes = [ctypes.POINTER(RefEnv)]
            getattr(L, f"fsph_ref_{pre}_destroy").argtypes = [vp]
            getattr(L, f"fsph_ref_{pre}_set").argtypes = [vp, ci, vp, vp]
            getattr(L, f"fsph_ref_{pre}_get").argtypes = [vp, ci, vp]
            getattr(L, f"fsph_ref_{pre}_scalars").argtypes = [vp, vp]
        L.fsph_ref_pbf_update.argtypes = [vp, cf, vp]
        L.fsph_ref_pbf_update.restype = ci
        L.fsph_ref_sph_update.argtypes = [vp, cf]
        L.fsph_ref_neighbors.argtypes = [vp, vp, ci, vp, vp, vp, ctypes.c_longlong]
        L.fsph_ref_neighbors.restype = ctypes.c_longlong
        L.fsph_ref_pbf_lambda.argtypes = [vp, vp, ci, cf, vp, vp]
        L.fsph_ref_pbf_dp.argtypes = [vp, vp, vp, ci, cf, vp]
        L.fsph_ref_pbf_predict.argtypes = [vp, cf, vp, vp, vp, vp]
        L.fsph_ref_sph_forces.argtypes = [vp, vp, vp, vp]
        L.fsph_ref_pbf_density_grid.argtypes = [vp, vp, ci, vp, vp, vp, vp]
        L.fsph_ref_cell_hash.argtypes = [vp, vp, ci, vp]
        L.fsph_ref_cell_hash.restype = ctypes.c_longlong
        L.fsph_ref_kernel.restype = cd
        L.fsph_ref_kernel.argtypes = [ci, cd, cd]
        L.fsph_ref_kernel_coef.restype = cd
        L.fsph_ref_kernel_coef.argtypes = [ci, cd]
        L.fsph_ref_wall.argtypes = [vp, vp, cd, vp, vp]
        L.fsph_ref_wall.restype = ci
        _ref = L
    return _ref


def ref_env_from_params(p, n: int) -> RefEnv:
    """Reference environment whose derived h / r / rho0 are overridden by the
    explicit values of an fsph_params (the reference derives them itself)."""
    e = RefEnv()
    e.max_particles = n
    for a in range(3):
        e.boundary_cen[a] = 0.5 * (p.box_min[a] + p.box_max[a])
        e.boundary_ext[a] = 0.5 * (p.box_max[a] - p.box_min[a])
    e.dens, e.mass, e.kernel_particles = p.rest_dens, p.mass, 20.0
    e.viscosity, e.gas_k = p.viscosity, p.gas_k
    e.epsilon, e.eta, e.min_iter, e.max_iter = p.epsilon, p.eta, p.min_iter, p.max_iter
    e.use_ap, e.ap_k, e.ap_n, e.ap_q = p.use_ap, p.ap_k, p.ap_n, p.ap_q
    e.h, e.particle_radius, e.rest_dens = p.h, p.particle_radius, p.rest_dens
    e.gravity_y = p.gravity[1]
    return e


class RefSolver:
    """The reference's rxPBDSPH (kind='pbf') or rxSPH (kind='sph'), CPU path."""

    def __init__(self, params, n: int, kind: str = "pbf"):
        self.L = ref_lib()
        if self.L is None:
            raise RuntimeError("reference CPU code unavailable (oracle/_ref not built)")
        self.kind = kind
        self.n = int(n)
        self.env = ref_env_from_params(params, self.n)
        self.h = getattr(self.L, f"fsph_ref_{kind}_create")(ctypes.byref(self.env))

    def __del__(self):
        if getattr(self, "h", None):
            getattr(self.L, f"fsph_ref_{self.kind}_destroy")(self.h)
            self.h = None

    def set(self, pos4, vel4=None):
        pos4 = _f4(pos4, self.n)
        vel4 = np.zeros_like(pos4) if vel4 is None else np.ascontiguousarray(vel4, dtype=np.float32)
        getattr(self.L, f"fsph_ref_{self.kind}_set")(self.h, self.n, _vp(pos4), _vp(vel4))

    def get(self, which: str) -> np.ndarray:
        if self.kind == "pbf":
            code = {"pos": 0, "vel": 1, "dens": 2, "lambda": 3, "dp": 4, "ppos": 5, "force": 6}[which]
            vec = which in ("pos", "vel", "dp", "ppos", "force")
        else:
            code = {"pos": 0, "vel": 1, "dens": 2, "pres": 3, "force": 4}[which]
            vec = which in ("pos", "vel", "force")
        out = np.zeros((self.n, 4) if vec else (self.n,), dtype=np.float32)
        getattr(self.L, f"fsph_ref_{self.kind}_get")(self.h, code, _vp(out))
        return out

    def scalars(self) -> np.ndarray:
        out = np.zeros(13, dtype=np.float64)
        getattr(self.L, f"fsph_ref_{self.kind}_scalars")(self.h, _vp(out))
        return out

    def update(self, dt: float):
        if self.kind == "pbf":
            eta = np.zeros(1, dtype=np.float64)
            it = self.L.fsph_ref_pbf_update(self.h, dt, _vp(eta))
            return it, float(eta[0])
        self.L.fsph_ref_sph_update(self.h, dt)
        return None

    def cell_hash(self, pos4):
        """rxNNGrid::CalGridHash(Vec3) of each position on the reference's CPU
        grid, and that grid's cell count."""
        pos4 = _f4(pos4, len(pos4))
        out = np.zeros(pos4.shape[0], np.uint32)
        cells = self.L.fsph_ref_cell_hash(self.h, _vp(pos4), pos4.shape[0], _vp(out))
        return out, int(cells)

    def neighbors(self, pos4):
        pos4 = _f4(pos4, self.n)
        off = np.zeros(self.n + 1, dtype=np.int32)
        cap = self.n * 80
        idx = np.zeros(cap, dtype=np.int32)
        d2 = np.zeros(cap, dtype=np.float32)
        t = self.L.fsph_ref_neighbors(self.h, _vp(pos4), self.n, _vp(off), _vp(idx), _vp(d2), cap)
        assert t <= cap
        return off, idx[:t], d2[:t]

    def lambda_pass(self, pos4, dt):
        pos4 = _f4(pos4, self.n)
        d = np.zeros(self.n, np.float32)
        l = np.zeros(self.n, np.float32)
        self.L.fsph_ref_pbf_lambda(self.h, _vp(pos4), self.n, dt, _vp(d), _vp(l))
        return d, l

    def correction_pass(self, pos4, lam, dt):
        pos4 = _f4(pos4, self.n)
        lam = np.ascontiguousarray(lam, dtype=np.float32)
        dp = np.zeros((self.n, 4), np.float32)
        self.L.fsph_ref_pbf_dp(self.h, _vp(pos4), _vp(lam), self.n, dt, _vp(dp))
        return dp

    def density_grid(self, pos4, n, minp, d):
        """rxPBDSPH::CalImplicitField of the given particles on an n[0] x n[1] x n[2]
        lattice from minp with spacing d; returns (n[2], n[1], n[0])."""
        pos4 = _f4(pos4, len(pos4))
        nn = np.ascontiguousarray(n, dtype=np.int32)
        out = np.zeros(int(np.prod(nn)), np.float32)
        self.L.fsph_ref_pbf_density_grid(self.h, _vp(pos4), pos4.shape[0], _vp(nn),
                                         _vp(np.ascontiguousarray(minp, np.float64)),
                                         _vp(np.ascontiguousarray(d, np.float64)), _vp(out))
        return out.reshape(nn[2], nn[1], nn[0])

    def sph_forces(self):
        d = np.zeros(self.n, np.float32)
        p = np.zeros(self.n, np.float32)
        a = np.zeros((self.n, 4), np.float32)
        self.L.fsph_ref_sph_forces(self.h, _vp(d), _vp(p), _vp(a))
        return d, p, a

    def pbf_predict(self, dt):
        d = np.zeros(self.n, np.float32)
        f = np.zeros((self.n, 4), np.float32)
        pp = np.zeros((self.n, 4), np.float32)
        pv = np.zeros((self.n, 4), np.float32)
        self.L.fsph_ref_pbf_predict(self.h, dt, _vp(d), _vp(f), _vp(pp), _vp(pv))
        return d, f, pp, pv


def csr_sets(off, idx):
    """Per-particle neighbour sets as sorted arrays (order-free comparison)."""
    return [np.sort(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]
