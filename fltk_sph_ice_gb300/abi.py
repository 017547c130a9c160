"""ctypes mirror of ``include/fsph.h`` and the loader of ``libfsph.so``.

The structs here must match the header field for field; ``tests/test_abi.py``
checks their sizes against the library's own ``sizeof`` report.  Loading is
strict: if the CUDA library has not been built, :func:`lib` raises -- there is
no CPU fallback behind this package.
"""
from __future__ import annotations

import ctypes
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
# FSPH_LIBRARY names another build of the same library to load instead (the
# bounds-checking debug build, fltk_sph_ice_gb300.build --debug-bounds)
LIB_PATH = os.environ.get("FSPH_LIBRARY") or os.path.join(PKG_DIR, "_build", "libfsph.so")

# fsph_status
OK, INVALID_ARG, OOM, CUDA_ERROR, NAN_DETECTED, TIMEOUT, NOT_CONVERGED, NOT_INITIALIZED, UNSUPPORTED, NO_DEVICE = range(10)
# fsph_solver
SOLVER_WCSPH, SOLVER_PBF = 0, 1
# fsph_error_mode
ERR_ONE_SIDED, ERR_TWO_SIDED = 0, 1
# fsph_where
HOST, DEVICE = 0, 1
BOUNDARY_POSITION, BOUNDARY_VOLUME, BOUNDARY_LAMBDA = 0, 1, 2
# fsph_array (numbering of rxParticleSystemBase::rxParticleArray, rx_ps.h:68-116)
RX_POSITION = 0
RX_VELOCITY = 1
RX_FORCE = 3
RX_DENSITY = 4
RX_PRESSURE = 5
RX_ATTRIBUTE = 7
RX_PREDICT_POS = 8
RX_PREDICT_VEL = 9
RX_SCALING_FACTOR = 10
RX_CORRECTION = 11
RX_STEP_CORRECTION = 12
RX_VORTICITY = 18
FSPH_SORTED_ID = 64
FSPH_FEATURES = 65

VECTOR_ARRAYS = {RX_POSITION, RX_VELOCITY, RX_FORCE, RX_PREDICT_POS, RX_PREDICT_VEL, RX_CORRECTION, RX_VORTICITY,
                 RX_STEP_CORRECTION}

# learned warm start (fsph.h)
MLP_FEATURES, MLP_HIDDEN, MLP_OUTPUTS, MLP_BLOB_SIZE = 32, 64, 3, 6532
WARM_NONE, WARM_LEARNED = 0, 1

STATUS_NAMES = {
    OK: "FSPH_OK", INVALID_ARG: "FSPH_INVALID_ARG", OOM: "FSPH_OOM", CUDA_ERROR: "FSPH_CUDA_ERROR",
    NAN_DETECTED: "FSPH_NAN_DETECTED", TIMEOUT: "FSPH_TIMEOUT", NOT_CONVERGED: "FSPH_NOT_CONVERGED",
    NOT_INITIALIZED: "FSPH_NOT_INITIALIZED", UNSUPPORTED: "FSPH_UNSUPPORTED", NO_DEVICE: "FSPH_NO_DEVICE",
}


class FsphParams(ctypes.Structure):
    _fields_ = [
        ("solver", ctypes.c_int),
        ("max_particles", ctypes.c_int),
        ("h", ctypes.c_float),
        ("mass", ctypes.c_float),
        ("rest_dens", ctypes.c_float),
        ("particle_radius", ctypes.c_float),
        ("box_min", ctypes.c_double * 3),
        ("box_max", ctypes.c_double * 3),
        ("gravity", ctypes.c_float * 3),
        ("viscosity", ctypes.c_float),
        ("gas_k", ctypes.c_float),
        ("epsilon", ctypes.c_float),
        ("eta", ctypes.c_float),
        ("min_iter", ctypes.c_int),
        ("max_iter", ctypes.c_int),
        ("error_mode", ctypes.c_int),
        ("use_ap", ctypes.c_int),
        ("ap_k", ctypes.c_float),
        ("ap_n", ctypes.c_float),
        ("ap_q", ctypes.c_float),
        ("xsph_c", ctypes.c_float),
        ("vort_eps", ctypes.c_float),
        ("cell_skin", ctypes.c_float),
        ("use_graph", ctypes.c_int),
        ("warm_start", ctypes.c_int),
        ("clamp_constraint", ctypes.c_int),
        ("walk_cells", ctypes.c_int),
        ("collect_features", ctypes.c_int),
        ("compensated_density", ctypes.c_int),
        ("grid_sort", ctypes.c_int),
        ("mlp_tcgen05", ctypes.c_int),
        ("reserved", ctypes.c_int * 1),
    ]

    def to_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if hasattr(v, "__len__") else v
        return d


class FsphEnv(ctypes.Structure):
    _fields_ = [
        ("solver", ctypes.c_int),
        ("max_particles", ctypes.c_int),
        ("boundary_cen", ctypes.c_double * 3),
        ("boundary_ext", ctypes.c_double * 3),
        ("dens", ctypes.c_float),
        ("mass", ctypes.c_float),
        ("kernel_particles", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("gas_k", ctypes.c_float),
        ("epsilon", ctypes.c_float),
        ("eta", ctypes.c_float),
        ("min_iter", ctypes.c_int),
        ("max_iter", ctypes.c_int),
        ("use_ap", ctypes.c_int),
        ("ap_k", ctypes.c_float),
        ("ap_n", ctypes.c_float),
        ("ap_q", ctypes.c_float),
        ("gravity_y", ctypes.c_float),
    ]


class FsphStepStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("grid_builds", ctypes.c_int),
        ("density_error", ctypes.c_float),
        ("density_error_one_sided", ctypes.c_float),
        ("density_error_two_sided", ctypes.c_float),
        ("density_error_max", ctypes.c_float),
        ("status", ctypes.c_int),
        ("kernels", ctypes.c_int),
        ("bounds_bits", ctypes.c_int),
        ("reserved", ctypes.c_int * 1),
    ]


class FsphBatchConfig(ctypes.Structure):
    _fields_ = [
        ("block", ctypes.c_int),
        ("lanes", ctypes.c_int),
        ("cell_skin", ctypes.c_float),
        ("eager", ctypes.c_int),
    ]


# Every symbol include/fsph.h declares (checked by tests/test_abi.py).
EXPORTS = [
    "fsph_abi_version", "fsph_status_string", "fsph_last_error", "fsph_params_from_env",
    "fsph_params_default", "fsph_create", "fsph_destroy", "fsph_set_params", "fsph_get_params",
    "fsph_num_particles", "fsph_set_particles", "fsph_set_array", "fsph_step", "fsph_last_stats",
    "fsph_get_array", "fsph_device_ptr", "fsph_sync", "fsph_neighbors", "fsph_pbf_eval_lambda",
    "fsph_pbf_eval_correction", "fsph_pbf_eval_xsph_vorticity", "fsph_sph_eval_forces", "fsph_time_pass",
    "fsph_pbf_eval_lambda_noalloc", "fsph_neighbors_ex", "fsph_step_fields",
    "fsph_set_box_obstacle", "fsph_set_sphere_obstacle", "fsph_move_sphere_obstacle", "fsph_get_sphere_obstacle_pos",
    "fsph_clear_obstacles", "fsph_num_obstacles", "fsph_density_grid", "fsph_num_active", "fsph_add_delete_region",
    "fsph_clear_delete_regions", "fsph_add_inlet_line", "fsph_clear_inlets", "fsph_emit_inlets",
    "fsph_set_step_log", "fsph_set_alloc_fault", "fsph_reference_cell_hash", "fsph_save_state", "fsph_load_state",
    "fsph_set_polygon_obstacle", "fsph_clear_polygon_obstacles", "fsph_num_polygon_triangles", "fsph_polygon_collide", "fsph_num_inlets",
    "fsph_mlp_create", "fsph_mlp_destroy", "fsph_mlp_set_blob", "fsph_mlp_get_blob", "fsph_mlp_last_error",
    "fsph_mlp_forward", "fsph_mlp_forward_tcgen05", "fsph_mlp_gradient", "fsph_mlp_train", "fsph_set_warm_start_model",
    "fsph_set_boundary", "fsph_num_boundary", "fsph_get_boundary",
    "fsph_batch_create", "fsph_batch_destroy", "fsph_batch_last_error", "fsph_batch_num_particles",
    "fsph_batch_offsets", "fsph_batch_set_particles", "fsph_batch_step", "fsph_batch_get_array",
    "fsph_batch_scene_stats", "fsph_batch_set_config", "fsph_batch_get_config", "fsph_batch_autotune",
]

# fsph_pass
PASS_LAMBDA, PASS_CORRECTION, PASS_GRID, PASS_LIST, PASS_SPH_DENSITY, PASS_SPH_FORCE = 0, 1, 2, 3, 4, 5

_LIB = None


def _declare(L: ctypes.CDLL) -> ctypes.CDLL:
    c_int, c_float, c_void_p, c_char_p = ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_char_p
    P = ctypes.POINTER
    L.fsph_abi_version.restype = c_int
    L.fsph_status_string.restype = c_char_p
    L.fsph_status_string.argtypes = [c_int]
    L.fsph_last_error.restype = c_char_p
    L.fsph_last_error.argtypes = [c_void_p]
    L.fsph_params_from_env.argtypes = [P(FsphEnv), P(FsphParams)]
    L.fsph_params_default.argtypes = [P(FsphParams)]
    L.fsph_params_default.restype = None
    L.fsph_create.argtypes = [P(FsphParams), P(c_void_p)]
    L.fsph_destroy.argtypes = [c_void_p]
    L.fsph_set_params.argtypes = [c_void_p, P(FsphParams)]
    L.fsph_get_params.argtypes = [c_void_p, P(FsphParams)]
    L.fsph_num_particles.argtypes = [c_void_p]
    L.fsph_set_particles.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_int]
    L.fsph_set_array.argtypes = [c_void_p, c_int, c_void_p, c_int, c_int, c_int]
    L.fsph_step.argtypes = [c_void_p, c_float, c_void_p, P(FsphStepStats)]
    L.fsph_last_stats.argtypes = [c_void_p, P(FsphStepStats)]
    L.fsph_get_array.argtypes = [c_void_p, c_int, c_void_p, c_int, c_void_p]
    L.fsph_device_ptr.argtypes = [c_void_p, c_int]
    L.fsph_device_ptr.restype = c_void_p
    L.fsph_sync.argtypes = [c_void_p]
    L.fsph_neighbors.argtypes = [c_void_p, c_void_p, c_void_p, ctypes.c_longlong, P(ctypes.c_longlong)]
    L.fsph_pbf_eval_lambda.argtypes = [c_void_p, c_void_p, c_int, c_void_p, c_void_p]
    L.fsph_pbf_eval_correction.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_float, c_void_p]
    L.fsph_sph_eval_forces.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]
    L.fsph_pbf_eval_xsph_vorticity.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float, c_void_p,
                                               c_void_p]
    L.fsph_neighbors_ex.argtypes = [c_void_p, c_void_p, c_int, c_float, c_int, c_void_p, c_void_p, c_void_p,
                                    ctypes.c_longlong, P(ctypes.c_longlong)]
    L.fsph_step_fields.argtypes = [c_void_p, c_float, c_void_p]
    L.fsph_set_box_obstacle.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]
    L.fsph_set_sphere_obstacle.argtypes = [c_void_p, c_void_p, ctypes.c_double, c_void_p, c_int]
    L.fsph_move_sphere_obstacle.argtypes = [c_void_p, c_int, c_void_p]
    L.fsph_get_sphere_obstacle_pos.argtypes = [c_void_p, c_int, c_void_p]
    L.fsph_clear_obstacles.argtypes = [c_void_p]
    L.fsph_num_obstacles.argtypes = [c_void_p]
    L.fsph_density_grid.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]
    L.fsph_num_active.argtypes = [c_void_p]
    L.fsph_add_delete_region.argtypes = [c_void_p, c_void_p, c_void_p]
    L.fsph_clear_delete_regions.argtypes = [c_void_p]
    L.fsph_add_inlet_line.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int,
                                      ctypes.c_double]
    L.fsph_clear_inlets.argtypes = [c_void_p]
    L.fsph_emit_inlets.argtypes = [c_void_p, c_int, P(c_int)]
    L.fsph_set_step_log.argtypes = [c_void_p, ctypes.c_char_p]
    L.fsph_save_state.argtypes = [c_void_p, ctypes.c_char_p]
    L.fsph_set_polygon_obstacle.argtypes = [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p]
    L.fsph_clear_polygon_obstacles.argtypes = [c_void_p]
    L.fsph_num_inlets.argtypes = [c_void_p]
    L.fsph_num_polygon_triangles.argtypes = [c_void_p]
    L.fsph_polygon_collide.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float, c_int]
    L.fsph_load_state.argtypes = [c_void_p, ctypes.c_char_p]
    L.fsph_reference_cell_hash.argtypes = [c_void_p, c_int, c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]
    L.fsph_set_alloc_fault.argtypes = [ctypes.c_longlong, ctypes.c_longlong]
    L.fsph_time_pass.argtypes = [c_void_p, c_int, c_int, P(c_float)]
    L.fsph_mlp_create.argtypes = [P(c_void_p)]
    L.fsph_mlp_destroy.argtypes = [c_void_p]
    L.fsph_mlp_set_blob.argtypes = [c_void_p, c_void_p]
    L.fsph_mlp_get_blob.argtypes = [c_void_p, c_void_p]
    L.fsph_mlp_last_error.argtypes = [c_void_p]
    L.fsph_mlp_last_error.restype = c_char_p
    L.fsph_mlp_forward.argtypes = [c_void_p, c_void_p, c_int, c_void_p, c_void_p]
    L.fsph_mlp_forward_tcgen05.argtypes = [c_void_p, c_void_p, c_int, c_void_p]
    L.fsph_mlp_gradient.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_void_p, P(c_float)]
    L.fsph_mlp_train.argtypes = [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_float, c_void_p]
    L.fsph_set_warm_start_model.argtypes = [c_void_p, c_void_p]
    L.fsph_set_boundary.argtypes = [c_void_p, c_void_p, c_int, c_int]
    L.fsph_set_boundary.restype = c_int
    L.fsph_num_boundary.argtypes = [c_void_p]
    L.fsph_num_boundary.restype = c_int
    L.fsph_get_boundary.argtypes = [c_void_p, c_int, c_void_p]
    L.fsph_get_boundary.restype = c_int
    L.fsph_batch_create.argtypes = [c_void_p, c_void_p, c_int, c_int, P(c_void_p)]
    L.fsph_batch_destroy.argtypes = [c_void_p]
    L.fsph_batch_last_error.argtypes = [c_void_p]
    L.fsph_batch_last_error.restype = c_char_p
    L.fsph_batch_num_particles.argtypes = [c_void_p]
    L.fsph_batch_offsets.argtypes = [c_void_p, c_void_p]
    L.fsph_batch_set_particles.argtypes = [c_void_p, c_void_p, c_void_p, c_int]
    L.fsph_batch_step.argtypes = [c_void_p, c_float, c_void_p]
    L.fsph_batch_get_array.argtypes = [c_void_p, c_int, c_void_p, c_int]
    L.fsph_batch_scene_stats.argtypes = [c_void_p, c_int, P(FsphStepStats)]
    L.fsph_batch_set_config.argtypes = [c_void_p, P(FsphBatchConfig)]
    L.fsph_batch_get_config.argtypes = [c_void_p, P(FsphBatchConfig)]
    L.fsph_batch_autotune.argtypes = [c_void_p, c_float, c_int, P(FsphBatchConfig), P(c_float)]
    for name in ["fsph_batch_create", "fsph_batch_destroy", "fsph_batch_num_particles", "fsph_batch_offsets",
                 "fsph_batch_set_particles", "fsph_batch_step", "fsph_batch_get_array", "fsph_batch_scene_stats",
                 "fsph_batch_set_config", "fsph_batch_get_config", "fsph_batch_autotune"]:
        getattr(L, name).restype = c_int
    for name in ["fsph_mlp_create", "fsph_mlp_destroy", "fsph_mlp_set_blob", "fsph_mlp_get_blob",
                 "fsph_mlp_forward", "fsph_mlp_forward_tcgen05", "fsph_mlp_gradient", "fsph_mlp_train",
                 "fsph_set_warm_start_model",
                 "fsph_time_pass", "fsph_create", "fsph_destroy", "fsph_set_params", "fsph_get_params", "fsph_num_particles",
                 "fsph_set_particles", "fsph_set_array", "fsph_step", "fsph_last_stats", "fsph_get_array",
                 "fsph_sync", "fsph_neighbors", "fsph_pbf_eval_lambda", "fsph_pbf_eval_correction",
                 "fsph_pbf_eval_xsph_vorticity", "fsph_sph_eval_forces", "fsph_params_from_env",
                 "fsph_neighbors_ex", "fsph_step_fields", "fsph_set_box_obstacle", "fsph_set_sphere_obstacle",
                 "fsph_move_sphere_obstacle", "fsph_get_sphere_obstacle_pos", "fsph_clear_obstacles",
                 "fsph_num_obstacles", "fsph_density_grid", "fsph_num_active", "fsph_add_delete_region",
                 "fsph_clear_delete_regions", "fsph_add_inlet_line", "fsph_clear_inlets", "fsph_emit_inlets",
                 "fsph_set_step_log", "fsph_set_alloc_fault", "fsph_reference_cell_hash", "fsph_save_state",
                 "fsph_load_state", "fsph_set_polygon_obstacle", "fsph_clear_polygon_obstacles",
                 "fsph_num_polygon_triangles", "fsph_polygon_collide", "fsph_num_inlets"]:
        getattr(L, name).restype = c_int
    return L


def lib(path: str | None = None) -> ctypes.CDLL:
    """Load libfsph.so (built by ``fltk_sph_ice_gb300.build``); raise if absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.isfile(p):
        raise RuntimeError(
            f"libfsph.so not found at {p}: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback")
    L = _declare(ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL))
    if path is None:
        _LIB = L
    return L


class FsphError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def set_alloc_fault(max_bytes: int = -1, fail_at: int = -1) -> None:
    """Device-allocation fault injection for tests (fsph_set_alloc_fault):
    refuse allocations above `max_bytes` and the `fail_at`-th allocation
    from now; (-1, -1) switches it off."""
    lib().fsph_set_alloc_fault(int(max_bytes), int(fail_at))
