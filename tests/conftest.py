import ctypes
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")


def cuda_device_count() -> int:
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    else:
        return 0
    n = ctypes.c_int(0)
    if rt.cudaGetDeviceCount(ctypes.byref(n)) != 0:
        return 0
    return n.value


@pytest.fixture(scope="session")
def fsph():
    """libfsph.so, built in-tree on first use."""
    from fltk_sph_ice_gb300 import abi, build
    build.build()
    return abi.lib()


@pytest.fixture(scope="session")
def gpu(fsph):
    if cuda_device_count() == 0:
        pytest.fail("no CUDA device: the gpu-marked tests need one (no CPU fallback exists)")
    return fsph


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def params_from_golden(g):
    from fltk_sph_ice_gb300 import abi
    return abi.FsphParams.from_buffer_copy(g["params"].tobytes())


def rel_err(a, b) -> float:
    """max |a - b| / max |b| over the whole field (norm-wise relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(float(np.abs(b).max()), 1e-300)
    return float(np.abs(a - b).max() / scale)


def assert_rel(a, b, tol, what=""):
    e = rel_err(a, b)
    assert e <= tol, f"{what}: max|a-b|/max|b| = {e:.3e} > {tol:.1e}"


def csr_rows(off, idx):
    return [np.sort(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def assert_same_sets(off_a, idx_a, off_b, idx_b):
    assert len(off_a) == len(off_b)
    ra, rb = csr_rows(off_a, idx_a), csr_rows(off_b, idx_b)
    bad = [i for i, (x, y) in enumerate(zip(ra, rb)) if not np.array_equal(x, y)]
    assert not bad, f"{len(bad)} particles with different neighbour sets, first {bad[:5]}"


def assert_close(a, b, what, tol=1e-5, etol=1e-4, floor=1e-2, atol=None):
    """Norm-wise: |a - b| <= tol max|b| + atol.  Element-wise, on the entries
    above floor max|b|: |a - b| <= etol |b| + atol.  atol (per entry): the
    FP32 storage error of the stored results a compared quantity is a
    difference of (e.g. a position change), else 0."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.abs(b).max()
    at = np.zeros(b.shape) if atol is None else np.broadcast_to(np.asarray(atol, np.float64), b.shape)
    err = np.abs(a - b) - at
    assert err.max() <= tol * scale, f"{what}: max(|a-b| - atol) / max|b| = {err.max() / scale:.3e} > {tol:.1e}"
    big = np.abs(b) > floor * scale
    assert big.any()
    excess = err[big] - etol * np.abs(b)[big]
    assert excess.max() <= 0.0, f"{what}: element-wise bar exceeded on {(excess > 0).sum()} of {big.sum()} entries"


def ulp32(x):
    """Spacing of float32 numbers at |x|: the rounding of a stored FP32 result."""
    return np.spacing(np.abs(np.asarray(x, np.float32))).astype(np.float64)
