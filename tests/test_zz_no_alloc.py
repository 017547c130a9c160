"""fsph_pbf_eval_lambda_noalloc: the lambda pass for callers that cannot let
the library allocate device memory (an application that owns the whole GPU
through its own pool, a real-time loop that must not allocate).  Called
through the C ABI with device buffers the test owns, and checked against the
context-based entry point fsph_pbf_eval_lambda on the same positions, twice
in a row (the shared scratch keeps the first call's contents), within the
parity tolerance of the other GPU tests (1e-5 in max|a-b| / max|b|).
Collected last on purpose: a failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest

from conftest import assert_rel
from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 65536


def cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.fail("libcudart not found")


class DeviceBuffer:
    """Device memory owned by the caller (the test), not by the library."""

    def __init__(self, rt, nbytes):
        self.rt = rt
        self.ptr = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(self.ptr), ctypes.c_size_t(nbytes)) == 0
        self.nbytes = nbytes

    def upload(self, a):
        a = np.ascontiguousarray(a)
        assert self.rt.cudaMemcpy(self.ptr, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), 1) == 0

    def download(self, shape, dtype):
        out = np.empty(shape, dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), self.ptr, ctypes.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.ptr)


def compressed(pos, f):
    out = pos.copy()
    c = out[:, :3].mean(0)
    out[:, :3] = (c + (out[:, :3] - c) * f).astype(np.float32)
    return out


def test_no_alloc_lambda_matches_context_entry_point(gpu):
    L = gpu
    L.fsph_pbf_eval_lambda_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]
    L.fsph_pbf_eval_lambda_noalloc.restype = ctypes.c_int
    rt = cudart()
    sc = scenes.pbf_double_dam_break(block=(12, 12, 24))
    p = sc.params
    n = sc.n
    states = [compressed(sc.pos, 0.97), compressed(sc.pos, 0.95)]
    bpos, bd, bl = DeviceBuffer(rt, n * 16), DeviceBuffer(rt, n * 4), DeviceBuffer(rt, n * 4)
    try:
        for k, x in enumerate(states):
            bpos.upload(x)
            free0, free1, total = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
            assert rt.cudaMemGetInfo(ctypes.byref(free0), ctypes.byref(total)) == 0
            st = L.fsph_pbf_eval_lambda_noalloc(ctypes.byref(p), bpos.ptr, n, bd.ptr, bl.ptr, None)
            assert st == abi.OK, f"call {k + 1}: {abi.STATUS_NAMES.get(st, st)}"
            assert rt.cudaDeviceSynchronize() == 0
            assert rt.cudaMemGetInfo(ctypes.byref(free1), ctypes.byref(total)) == 0
            if k > 0:  # after the first call (module and scratch set-up) no device memory is taken
                assert free1.value == free0.value
            d = bd.download(n, np.float32)
            lam = bl.download(n, np.float32)
            ps = rxPBDSPH(p)
            d_ref, lam_ref = ps.EvalScalingFactor(x)
            ps.close()
            assert np.abs(lam_ref).max() > 0
            assert_rel(d, d_ref, 1e-5, f"density, call {k + 1}")
            assert_rel(lam, lam_ref, 1e-5, f"lambda, call {k + 1}")
        # sizes beyond the stated maximum are rejected before any launch
        st = L.fsph_pbf_eval_lambda_noalloc(ctypes.byref(p), bpos.ptr, MAX_PARTICLES + 1, bd.ptr, bl.ptr, None)
        assert st == abi.INVALID_ARG
        big = abi.FsphParams.from_buffer_copy(p)
        for a in range(3):
            big.box_max[a] = big.box_min[a] + 20.0  # about 430^3 cells, far more than 2^20
        st = L.fsph_pbf_eval_lambda_noalloc(ctypes.byref(big), bpos.ptr, n, bd.ptr, bl.ptr, None)
        assert st == abi.INVALID_ARG
    finally:
        for b in (bpos, bd, bl):
            b.free()
