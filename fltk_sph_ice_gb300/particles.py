"""Python mirror of the reference's particle-system operator surface.

rxParticleSystemBase (rx_ps.h:55-333) with its concrete solvers rxSPH
(WCSPH, rx_sph.h:202-426) and rxPBDSPH (PBF, rx_sph.h:1027-1274): the same
method names and meanings (Set, Update, GetArrayVBO, SetArrayVBO,
SetParticlesToCell / GetNeights, SetGravity, SetIterations ...), implemented
over the C ABI of libfsph.so (include/fsph.h).  Errors raise FsphError with
the library's status and message; nothing here computes physics.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from . import abi
from .abi import FsphError


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class rxParticleSystemBase:
    """One GPU fluid context (fsph_ctx)."""

    solver = abi.SOLVER_PBF

    def __init__(self, params: abi.FsphParams):
        self.L = abi.lib()
        p = abi.FsphParams.from_buffer_copy(params)
        p.solver = self.solver
        self._ctx = ctypes.c_void_p()
        st = self.L.fsph_create(ctypes.byref(p), ctypes.byref(self._ctx))
        if st != abi.OK:
            raise FsphError(st, "fsph_create failed")
        self.last_stats = abi.FsphStepStats()

    # -- lifetime -------------------------------------------------------
    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            self.L.fsph_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int, what: str):
        if st != abi.OK:
            msg = self.L.fsph_last_error(self._ctx)
            raise FsphError(st, f"{what}: {msg.decode() if msg else ''}")

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._ctx

    # -- Initialize / parameters -----------------------------------------
    @classmethod
    def from_env(cls, env: abi.FsphEnv):
        """rxPBDSPH::Initialize / rxSPH::Initialize derivation from a scene env."""
        p = abi.FsphParams()
        L = abi.lib()
        e = abi.FsphEnv.from_buffer_copy(env)
        e.solver = cls.solver
        st = L.fsph_params_from_env(ctypes.byref(e), ctypes.byref(p))
        if st != abi.OK:
            raise FsphError(st, "fsph_params_from_env")
        return cls(p)

    def GetParams(self) -> abi.FsphParams:
        p = abi.FsphParams()
        self._check(self.L.fsph_get_params(self._ctx, ctypes.byref(p)), "fsph_get_params")
        return p

    def SetParams(self, p: abi.FsphParams):
        q = abi.FsphParams.from_buffer_copy(p)
        q.solver = self.solver
        self._check(self.L.fsph_set_params(self._ctx, ctypes.byref(q)), "fsph_set_params")

    def SetGravity(self, g: float):
        """rx_ps.h:227 -- gravity (0, g, 0)."""
        p = self.GetParams()
        p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, g, 0.0
        self.SetParams(p)

    def SetIterations(self, i: int):
        """rx_ps.h:220 -- solver iteration cap."""
        p = self.GetParams()
        p.max_iter = int(i)
        self.SetParams(p)

    def GetNumParticles(self) -> int:
        return int(self.L.fsph_num_particles(self._ctx))

    def GetMaxParticles(self) -> int:
        return int(self.GetParams().max_particles)

    def GetParticleRadius(self) -> float:
        return float(self.GetParams().particle_radius)

    # -- particle data ---------------------------------------------------
    def Set(self, pos, vel=None) -> bool:
        """rxParticleSystemBase::Set (rx_ps.cpp:30-59); pos/vel (N,3) or (N,4)."""
        pos4 = _as4(pos)
        vel4 = None if vel is None else _as4(vel)
        self._check(self.L.fsph_set_particles(self._ctx, _ptr(pos4), _ptr(vel4), pos4.shape[0], abi.HOST),
                    "fsph_set_particles")
        return True

    def SetArrayVBO(self, type_: int, data, start: int = 0, count: int | None = None):
        """SetArrayVBO (rx_ps.h:260-262): overwrite `count` particles from `start`."""
        if type_ == abi.RX_ATTRIBUTE:
            arr = np.ascontiguousarray(data, dtype=np.int32).reshape(-1)
        else:
            arr = _as4(data)
        n = arr.shape[0] if count is None else int(count)
        self._check(self.L.fsph_set_array(self._ctx, type_, _ptr(arr), int(start), n, abi.HOST), "fsph_set_array")

    def GetArrayVBO(self, type_: int, d2h: bool = True) -> np.ndarray:
        """GetArrayVBO (rx_ps.h:259): a copy of one array in particle order."""
        n = self.GetNumParticles()
        if type_ == abi.FSPH_FEATURES:
            out = np.zeros((n, abi.MLP_FEATURES), dtype=np.float32)
        elif type_ in abi.VECTOR_ARRAYS:
            out = np.zeros((n, 4), dtype=np.float32)
        elif type_ in (abi.RX_ATTRIBUTE, abi.FSPH_SORTED_ID):
            out = np.zeros(n, dtype=np.int32)
        else:
            out = np.zeros(n, dtype=np.float32)
        if n:
            self._check(self.L.fsph_get_array(self._ctx, type_, _ptr(out), abi.HOST, None), "fsph_get_array")
        return out

    def GetParticle(self) -> np.ndarray:
        return self.GetArrayVBO(abi.RX_POSITION)

    def GetParticleDevice(self) -> int:
        """Borrowed device pointer (device order) to the positions."""
        return int(self.L.fsph_device_ptr(self._ctx, abi.RX_POSITION) or 0)

    # -- step ------------------------------------------------------------
    def Update(self, dt: float, step: int = 0, stats: bool = True) -> bool:
        """rxParticleSystemBase::Update (rx_ps.h:254): the inlet lines due at
        `step` emit their particles (rx_sph_pbd_gpu.cpp:795-815), then one step."""
        if getattr(self, "_inlets", 0):
            self._check(self.L.fsph_emit_inlets(self._ctx, int(step), None), "fsph_emit_inlets")
        st = self.L.fsph_step(self._ctx, float(dt), None, ctypes.byref(self.last_stats) if stats else None)
        self._check(st, "fsph_step")
        return True

    # -- dynamic particle count: inlets and deletion regions ---------------
    def AddLine(self, pos1, pos2, vel, up, accum: int, span: int, spacing: float) -> int:
        """An inlet line (rxInletLine / AddLine, rx_ps.h:41-49, rx_ps.cpp:432)."""
        d = lambda v: np.ascontiguousarray(v, dtype=np.float64)  # noqa: E731
        a, b, v, u = d(pos1), d(pos2), d(vel), d(up)
        k = self.L.fsph_add_inlet_line(self._ctx, _ptr(a), _ptr(b), _ptr(v), _ptr(u), int(accum), int(span),
                                       float(spacing))
        if k <= 0:  # a negated status
            self._check(-k if k else abi.INVALID_ARG, "fsph_add_inlet_line")
        self._inlets = k
        return k

    def EmitInlets(self, step: int) -> int:
        """The particles of the inlet lines due at `step`; returns how many."""
        n = ctypes.c_int(0)
        self._check(self.L.fsph_emit_inlets(self._ctx, int(step), ctypes.byref(n)), "fsph_emit_inlets")
        return n.value

    def AddDeleteRegion(self, lo, hi):
        """Particles strictly inside [lo, hi] at the end of a step are deleted
        (attribute -1, parked far away; env.delete_region, rx_sph.h:125-126)."""
        a, b = np.ascontiguousarray(lo, np.float64), np.ascontiguousarray(hi, np.float64)
        self._check(self.L.fsph_add_delete_region(self._ctx, _ptr(a), _ptr(b)), "fsph_add_delete_region")

    def GetNumActiveParticles(self) -> int:
        return int(self.L.fsph_num_active(self._ctx))

    def SaveState(self, path: str):
        """The exact device state (fsph_save_state): resuming from it with
        LoadState steps bit-identically to continuing."""
        self._check(self.L.fsph_save_state(self._ctx, os.fsencode(path)), "fsph_save_state")

    def LoadState(self, path: str):
        self._check(self.L.fsph_load_state(self._ctx, os.fsencode(path)), "fsph_load_state")
        self._inlets = int(self.L.fsph_num_inlets(self._ctx))  # the state's inlet lines emit from here on

    def OutputParticles(self, path: str):
        """The reference's particle file (rx_ps.cpp:581-612): uint32 N, N x 3
        float32 positions, N x 3 float32 velocities."""
        x = self.GetArrayVBO(abi.RX_POSITION)[:, :3]
        v = self.GetArrayVBO(abi.RX_VELOCITY)[:, :3]
        with open(path, "wb") as f:
            f.write(np.uint32(x.shape[0]).tobytes())
            f.write(np.ascontiguousarray(x, np.float32).tobytes())
            f.write(np.ascontiguousarray(v, np.float32).tobytes())

    def InputParticles(self, path: str):
        """rx_ps.cpp:614-644: the positions (and velocities, when present) of
        a particle file replace the current particles."""
        raw = open(path, "rb").read()
        n = int(np.frombuffer(raw[:4], np.uint32)[0])
        body = np.frombuffer(raw[4:], np.float32)
        if body.size < 3 * n:
            raise ValueError("particle file truncated")
        x = body[:3 * n].reshape(n, 3)
        v = body[3 * n:6 * n].reshape(n, 3) if body.size >= 6 * n else None
        self.Set(x, v)

    def SaveCheckpoint(self, path: str, seed: int | None = None):
        """Particle file at `path`, exact state at path + '.state', JSON
        sidecar at path + '.json' (parameters, counts, the scene seed)."""
        self.OutputParticles(path)
        self.SaveState(path + ".state")
        side = {"format": "fsph checkpoint 1", "params": self.GetParams().to_dict(), "seed": seed,
                "particles": self.GetNumParticles(), "active": self.GetNumActiveParticles(),
                "state": os.path.basename(path) + ".state",
                "jitter": "inlet jitter is counter-based on (line, step); no generator state"}
        with open(path + ".json", "w") as f:
            json.dump(side, f, indent=1)

    def LoadCheckpoint(self, path: str):
        """Resume from SaveCheckpoint's files; returns the sidecar's seed."""
        with open(path + ".json") as f:
            side = json.load(f)
        st = path + ".state"
        if os.path.isfile(st):
            self.LoadState(st)
        else:
            self.InputParticles(path)
        return side.get("seed")

    def SetStepLog(self, path: str | None):
        """Append one JSON line per step to `path` (None stops the log)."""
        self._check(self.L.fsph_set_step_log(self._ctx, path.encode() if path else None), "fsph_set_step_log")

    def Sync(self):
        self._check(self.L.fsph_sync(self._ctx), "fsph_sync")

    def LastStats(self) -> abi.FsphStepStats:
        self._check(self.L.fsph_last_stats(self._ctx, ctypes.byref(self.last_stats)), "fsph_last_stats")
        return self.last_stats

    # -- neighbours --------------------------------------------------------
    def SetParticlesToCell(self, prts=None, h: float = -1.0):
        """SetParticlesToCell() / (prts, n, h) (rx_sph_pbd.cpp:1735-1750): the
        neighbour sets of the current particles, or of the given positions
        among themselves, within h (default: the kernel radius), kept for
        GetNeights.  Returns CSR (offsets[n+1], indices ascending in each row,
        dist2 = each pair's squared distance as the reference's rxNeigh::Dist2)."""
        p4 = None if prts is None else _as4(prts)
        n = self.GetNumParticles() if p4 is None else p4.shape[0]
        off = np.zeros(n + 1, dtype=np.int32)
        total = ctypes.c_longlong(0)
        self._check(self.L.fsph_neighbors_ex(self._ctx, _ptr(p4), n, float(h), abi.HOST, _ptr(off), None, None, 0,
                                             ctypes.byref(total)), "fsph_neighbors_ex")
        idx = np.zeros(max(total.value, 1), dtype=np.int32)
        d2 = np.zeros(max(total.value, 1), dtype=np.float32)
        self._check(self.L.fsph_neighbors_ex(self._ctx, _ptr(p4), n, float(h), abi.HOST, _ptr(off), _ptr(idx),
                                             _ptr(d2), total.value, ctypes.byref(total)), "fsph_neighbors_ex")
        self._neighs = (off, idx[:total.value], d2[:total.value])
        return self._neighs

    def GetNeights(self):
        """Neighbour sets of the current positions (GetNeights, rx_sph.h:1196) as
        CSR (offsets[n+1], indices), particle indices ascending in each row."""
        n = self.GetNumParticles()
        off = np.zeros(n + 1, dtype=np.int32)
        total = ctypes.c_longlong(0)
        self._check(self.L.fsph_neighbors(self._ctx, _ptr(off), None, 0, ctypes.byref(total)), "fsph_neighbors")
        idx = np.zeros(max(total.value, 1), dtype=np.int32)
        self._check(self.L.fsph_neighbors(self._ctx, _ptr(off), _ptr(idx), total.value, ctypes.byref(total)),
                    "fsph_neighbors")
        return off, idx[:total.value]

    # -- density on a lattice (rx_ps.h:283-285) ----------------------------
    def CalGridHash(self, pos, rule: int = 0):
        """The reference's cell hash of each position: rule 0 = its CPU grid
        (rxNNGrid::CalGridHash), 1 = its GPU grid (calcGridPos /
        calcGridHash).  Returns (hash uint32[n], grid dims (3,), cell width)."""
        p4 = _as4(pos)
        out = np.zeros(p4.shape[0], np.uint32)
        g = np.zeros(3, np.int32)
        cw = ctypes.c_double()
        self._check(self.L.fsph_reference_cell_hash(self._ctx, int(rule), _ptr(p4), p4.shape[0], abi.HOST, _ptr(out),
                                                    _ptr(g), ctypes.byref(cw)), "fsph_reference_cell_hash")
        return out, g, cw.value

    def CalImplicitField(self, n, minp, d) -> np.ndarray:
        """The density field of the current particles on an n[0] x n[1] x n[2]
        lattice from minp with spacing d (CalImplicitField, rx_sph_pbd.cpp:2036):
        an (n[2], n[1], n[0]) float32 array, 0 outside the simulation range."""
        nn = np.ascontiguousarray(n, dtype=np.int32)
        out = np.zeros(int(np.prod(nn)), np.float32)
        self._check(self.L.fsph_density_grid(self._ctx, _ptr(nn), _ptr(np.ascontiguousarray(minp, np.float64)),
                                             _ptr(np.ascontiguousarray(d, np.float64)), _ptr(out), abi.HOST),
                    "fsph_density_grid")
        return out.reshape(nn[2], nn[1], nn[0])

    def GetImplicit(self, x: float, y: float, z: float) -> float:
        """The density field at one point (GetImplicit, rx_sph_pbd.cpp:2024)."""
        return float(self.CalImplicitField((1, 1, 1), (x, y, z), (1.0, 1.0, 1.0))[0, 0, 0])

    # -- analytic obstacles (rx_ps.h:266-272) ------------------------------
    def SetBoxObstacle(self, cen, ext, ang=(0.0, 0.0, 0.0), vel=(0.0, 0.0, 0.0), flg: int = 1):
        """A box obstacle: centre, half extents, Euler angles in degrees."""
        d = lambda v: np.ascontiguousarray(v, dtype=np.float64)  # noqa: E731
        c, e, a, v = d(cen), d(ext), d(ang), d(vel)
        self._check(self.L.fsph_set_box_obstacle(self._ctx, _ptr(c), _ptr(e), _ptr(a), _ptr(v), int(flg)),
                    "fsph_set_box_obstacle")

    def SetSphereObstacle(self, cen, rad: float, vel=(0.0, 0.0, 0.0), flg: int = 1):
        c, v = np.ascontiguousarray(cen, np.float64), np.ascontiguousarray(vel, np.float64)
        self._check(self.L.fsph_set_sphere_obstacle(self._ctx, _ptr(c), float(rad), _ptr(v), int(flg)),
                    "fsph_set_sphere_obstacle")

    def SetPolygonObstacle(self, vrts, nrms, tris, vel=(0.0, 0.0, 0.0)):
        """A triangle-mesh obstacle (rx_ps.h:268): vertices (nv, 3), normals
        (unused, as in the reference's collision), triangles (nt, 3)."""
        v = np.ascontiguousarray(vrts, np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
        w = np.ascontiguousarray(vel, np.float64)
        self._check(self.L.fsph_set_polygon_obstacle(self._ctx, _ptr(v), v.shape[0], _ptr(t), t.shape[0], _ptr(w)),
                    "fsph_set_polygon_obstacle")

    def ClearPolygonObstacles(self):
        self._check(self.L.fsph_clear_polygon_obstacles(self._ctx), "fsph_clear_polygon_obstacles")

    def GetNumPolygonTriangles(self) -> int:
        return int(self.L.fsph_num_polygon_triangles(self._ctx))

    def PolygonCollide(self, x0, x1, v, dt: float):
        """The triangle-mesh collision of the segments x0 -> x1 with velocities
        v: returns the updated (x1, v), (n, 4) float32."""
        a, b, c = _as4(x0), _as4(x1).copy(), _as4(v).copy()
        self._check(self.L.fsph_polygon_collide(self._ctx, _ptr(a), _ptr(b), _ptr(c), a.shape[0], float(dt), abi.HOST),
                    "fsph_polygon_collide")
        return b, c

    def MoveSphereObstacle(self, b: int, disp):
        d = np.ascontiguousarray(disp, np.float64)
        self._check(self.L.fsph_move_sphere_obstacle(self._ctx, int(b), _ptr(d)), "fsph_move_sphere_obstacle")

    def GetSphereObstaclePos(self, b: int = 0) -> np.ndarray:
        out = np.zeros(3, np.float64)
        self._check(self.L.fsph_get_sphere_obstacle_pos(self._ctx, int(b), _ptr(out)), "fsph_get_sphere_obstacle_pos")
        return out

    def ClearObstacles(self):
        self._check(self.L.fsph_clear_obstacles(self._ctx), "fsph_clear_obstacles")

    def UpdateWithoutPosAndVel(self, dt: float, step: int = 0) -> bool:
        """A step's fields without moving the particles (rx_ps.h:254,
        rx_sph_gpu.cpp:925): density, pressure and acceleration (WCSPH) or the
        PBF pre-pass density and external + viscous acceleration."""
        self._check(self.L.fsph_step_fields(self._ctx, float(dt), None), "fsph_step_fields")
        return True


class rxSPH(rxParticleSystemBase):
    """WCSPH solver (rxSPH / rxSPH_GPU)."""

    solver = abi.SOLVER_WCSPH

    def EvalForces(self, pos, vel):
        """calDensity + calForce on the given state (rx_sph_cpu.cpp:495-656)."""
        pos4, vel4 = _as4(pos), _as4(vel)
        n = pos4.shape[0]
        d = np.zeros(n, np.float32)
        p = np.zeros(n, np.float32)
        a = np.zeros((n, 4), np.float32)
        self._check(self.L.fsph_sph_eval_forces(self._ctx, _ptr(pos4), _ptr(vel4), n, _ptr(d), _ptr(p), _ptr(a)),
                    "fsph_sph_eval_forces")
        return d, p, a


class rxPBDSPH(rxParticleSystemBase):
    """PBF solver (rxPBDSPH / rxPBDSPH_GPU)."""

    solver = abi.SOLVER_PBF

    def SetBoundary(self, bpos):
        """Static boundary particles (the boundary set-up of rxPBDSPH::Initialize,
        rx_sph_pbd.cpp:280-297); bpos (NB,3) or (NB,4); an empty array removes them."""
        b4 = _as4(bpos) if len(bpos) else np.zeros((0, 4), np.float32)
        self._check(self.L.fsph_set_boundary(self._ctx, _ptr(b4) if b4.shape[0] else None, b4.shape[0], abi.HOST),
                    "fsph_set_boundary")

    def SetWarmStartModel(self, blob):
        """Install a trained warm-start network (FSPH_MLP_BLOB_SIZE floats);
        used by steps with params.warm_start = 1.  No counterpart in the
        reference (its PBF loop starts from the prediction, rx_sph_pbd.cpp:418-425)."""
        b = np.ascontiguousarray(blob, dtype=np.float32)
        if b.size != abi.MLP_BLOB_SIZE:
            raise ValueError(f"a network blob has {abi.MLP_BLOB_SIZE} floats")
        self._check(self.L.fsph_set_warm_start_model(self._ctx, _ptr(b)), "fsph_set_warm_start_model")

    def GetNumBoundaryParticles(self) -> int:
        return int(self.L.fsph_num_boundary(self._ctx))

    def GetBoundary(self, which: int) -> np.ndarray:
        """abi.BOUNDARY_POSITION (NB,4), BOUNDARY_VOLUME psi_b (NB,) or BOUNDARY_LAMBDA (NB,)."""
        nb = self.GetNumBoundaryParticles()
        out = np.zeros((nb, 4) if which == abi.BOUNDARY_POSITION else (nb,), np.float32)
        if nb:
            self._check(self.L.fsph_get_boundary(self._ctx, which, _ptr(out)), "fsph_get_boundary")
        return out

    def EvalScalingFactor(self, pos):
        """calScalingFactor on the given predicted positions (rx_sph_pbd.cpp:699-914)."""
        pos4 = _as4(pos)
        n = pos4.shape[0]
        d = np.zeros(n, np.float32)
        lam = np.zeros(n, np.float32)
        self._check(self.L.fsph_pbf_eval_lambda(self._ctx, _ptr(pos4), n, _ptr(d), _ptr(lam)),
                    "fsph_pbf_eval_lambda")
        return d, lam

    def EvalPositionCorrection(self, pos, lam, dt: float):
        """calPositionCorrection (rx_sph_pbd.cpp:925-1026)."""
        pos4 = _as4(pos)
        lam = np.ascontiguousarray(lam, dtype=np.float32)
        n = pos4.shape[0]
        dp = np.zeros((n, 4), np.float32)
        self._check(self.L.fsph_pbf_eval_correction(self._ctx, _ptr(pos4), _ptr(lam), n, float(dt), _ptr(dp)),
                    "fsph_pbf_eval_correction")
        return dp

    def EvalXsphVorticity(self, pos, vel, dens, dt: float):
        """The end-of-step XSPH smoothing (rx_pbdsph_kernel.cu:1090-1162) and
        vorticity confinement on the given state: (velocity after both, omega)."""
        pos4, vel4 = _as4(pos), _as4(vel)
        dens = np.ascontiguousarray(dens, dtype=np.float32)
        n = pos4.shape[0]
        vo = np.zeros((n, 4), np.float32)
        om = np.zeros((n, 4), np.float32)
        self._check(self.L.fsph_pbf_eval_xsph_vorticity(self._ctx, _ptr(pos4), _ptr(vel4), _ptr(dens), n, float(dt),
                                                        _ptr(vo), _ptr(om)), "fsph_pbf_eval_xsph_vorticity")
        return vo, om


def _as4(a) -> np.ndarray:
    a = np.asarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] not in (3, 4):
        raise ValueError("expected an (N, 3) or (N, 4) array")
    if a.shape[1] == 3:
        b = np.zeros((a.shape[0], 4), dtype=np.float32)
        b[:, :3] = a
        a = b
    return np.ascontiguousarray(a)
