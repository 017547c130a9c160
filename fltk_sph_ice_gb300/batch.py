"""Batched PBF scenes over the fsph_batch_* C ABI.

Many independent scenes of uneven particle counts advance together: each
pass of a step is one persistent launch over all scenes, the step is one
CUDA graph, and the launch shape (threads per block, lanes per particle in
the constraint passes, cell skin) is chosen by the library's autotuner.
Each scene behaves as its own rxPBDSPH::Update (rx_sph_pbd.cpp:377-484)
run for a fixed number of constraint iterations.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi


def _vp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class PBFBatch:
    """scenes: a list of (fsph_params, particle count); arrays cross this
    interface scene after scene (see `offsets`)."""

    def __init__(self, params: list, counts: list[int], iterations: int = 4):
        self._L = abi.lib()
        n = len(params)
        arr = (abi.FsphParams * n)(*params)
        cnt = np.ascontiguousarray(counts, dtype=np.int32)
        h = ctypes.c_void_p()
        st = self._L.fsph_batch_create(ctypes.cast(arr, ctypes.c_void_p), _vp(cnt), n, iterations, ctypes.byref(h))
        if st != abi.OK:
            raise abi.FsphError(st, "fsph_batch_create")
        self.handle = h
        self.nscenes = n
        off = np.zeros(n + 1, dtype=np.int32)
        self._check(self._L.fsph_batch_offsets(self.handle, _vp(off)))
        self.offsets = off
        self.n = int(off[-1])

    def _check(self, st: int):
        if st != abi.OK:
            msg = self._L.fsph_batch_last_error(self.handle).decode() if self.handle else ""
            raise abi.FsphError(st, msg)

    def close(self):
        if getattr(self, "handle", None):
            self._L.fsph_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, pos: np.ndarray, vel: np.ndarray | None = None):
        p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 4)
        if p.shape[0] != self.n:
            raise ValueError(f"expected {self.n} particles, got {p.shape[0]}")
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 4)
        self._check(self._L.fsph_batch_set_particles(self.handle, _vp(p), None if v is None else _vp(v), abi.HOST))

    def step(self, dt: float, stream=None):
        self._check(self._L.fsph_batch_step(self.handle, ctypes.c_float(dt), stream))

    def get(self, which: int) -> np.ndarray:
        if which == abi.RX_DENSITY:
            out = np.zeros(self.n, dtype=np.float32)
        else:
            out = np.zeros((self.n, 4), dtype=np.float32)
        self._check(self._L.fsph_batch_get_array(self.handle, which, _vp(out), abi.HOST))
        return out

    def scene(self, arr: np.ndarray, s: int) -> np.ndarray:
        return arr[self.offsets[s]:self.offsets[s + 1]]

    def scene_stats(self, s: int) -> abi.FsphStepStats:
        st = abi.FsphStepStats()
        self._check(self._L.fsph_batch_scene_stats(self.handle, s, ctypes.byref(st)))
        return st

    @property
    def config(self) -> abi.FsphBatchConfig:
        c = abi.FsphBatchConfig()
        self._check(self._L.fsph_batch_get_config(self.handle, ctypes.byref(c)))
        return c

    def set_config(self, block: int, lanes: int, cell_skin: float, eager: bool = False):
        c = abi.FsphBatchConfig(block, lanes, cell_skin, 1 if eager else 0)
        self._check(self._L.fsph_batch_set_config(self.handle, ctypes.byref(c)))

    def autotune(self, dt: float, steps: int = 3):
        """Time every candidate configuration from the current state (which is
        restored), install the fastest; returns (config, ms per step), ms = -1
        when the process-wide cache already held this scene set."""
        c = abi.FsphBatchConfig()
        ms = ctypes.c_float(0)
        self._check(self._L.fsph_batch_autotune(self.handle, ctypes.c_float(dt), steps, ctypes.byref(c),
                                                ctypes.byref(ms)))
        return c, float(ms.value)
