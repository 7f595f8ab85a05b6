"""ctypes binding of libpcd_gb300.so (the C ABI declared in include/pcd.h).

The library is loaded from the package's in-tree _build/ folder.  There is no
CPU fallback: when the library is missing, or no CUDA device is present, the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

PCD_OK = 0
PCD_NOT_CONVERGED = 1
PCD_BAD_ARG = 2
PCD_DEVICE_ERROR = 3
PCD_TIMEOUT = 4
PCD_RASTER_MISS = 5
PCD_NO_DEVICE = 6
PCD_FALLBACK_USED = 7
PCD_MESH_SMOOTHED = 8

STOP_MAX_UPDATE = 0
STOP_REL_RESIDUAL = 1
PREC_FP64 = 0
PREC_MIXED = 1
SCHED_AUTO = 0
SCHED_LAUNCHES = 1
SCHED_PERSISTENT = 2
SCHED_CLUSTER = 3
SCHED_STRIPES = 4
SCHED_STREAM = 5
SCHED_TILES = 6
SCHED_BLOCKS = 7
WARM_ZERO = 0
WARM_GIVEN = 1
WARM_LEARNED = 2


class PCDError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        super().__init__(f"{where}: status {status} ({status_string(status)}): {detail}")
        self.status = status


class SolveOpts(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int),
        ("tol", C.c_double),
        ("stop", C.c_int),
        ("precision", C.c_int),
        ("omega", C.c_double),
        ("check_every", C.c_int),
        ("refine_every", C.c_int),
        ("warm_start", C.c_int),
        ("schedule", C.c_int),
        ("refine_drop", C.c_double),
        ("block_sweeps", C.c_int),
    ]


class SolveStats(C.Structure):
    _fields_ = [
        ("sweeps", C.c_int),
        ("converged", C.c_int),
        ("rel_residual", C.c_double),
        ("max_residual", C.c_double),
        ("last_max_update", C.c_double),
        ("device_ms", C.c_double),
        ("residual_checks", C.c_int),
        ("sweep_ms", C.c_double),
        ("schedule_used", C.c_int),
        ("warm_used", C.c_int),
        ("warm_rel_residual", C.c_double),
        ("tuned", C.c_int),
        ("check_every_used", C.c_int),
        ("refine_every_used", C.c_int),
        ("refine_drop_used", C.c_double),
        ("warm_zero_rel_residual", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class DesignParams(C.Structure):
    _fields_ = [
        ("mesh_res_x", C.c_int),
        ("mesh_res_y", C.c_int),
        ("res_x", C.c_int),
        ("res_y", C.c_int),
        ("width", C.c_double),
        ("height", C.c_double),
        ("focal_l", C.c_double),
        ("thickness", C.c_double),
        ("transport", SolveOpts),
        ("height_solve", SolveOpts),
        ("raster_miss_policy", C.c_int),
    ]


class Instance(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("ld", C.c_int), ("b", C.c_void_p), ("phi", C.c_void_p)]


class InstanceStats(C.Structure):
    _fields_ = [("sweeps", C.c_int), ("converged", C.c_int), ("rel_residual", C.c_double), ("cycles", C.c_int)]


class BatchStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("clusters", C.c_int), ("cluster_size", C.c_int),
                ("smem_bytes", C.c_longlong), ("cell_sweeps", C.c_longlong), ("check_every", C.c_int),
                ("refine_drop", C.c_double), ("tuned", C.c_int)]


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol declared in include/pcd.h
SIGNATURES = {
    "pcd_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "pcd_ctx_destroy": (C.c_int, [_vp]),
    "pcd_ctx_stream": (_vp, [_vp]),
    "pcd_last_error": (C.c_char_p, []),
    "pcd_status_string": (C.c_char_p, [C.c_int]),
    "pcd_solve_opts_default": (C.c_int, [C.POINTER(SolveOpts)]),
    "pcd_kernel_launches": (C.c_ulonglong, []),
    "pcd_poisson_solver": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]),
    "pcd_poisson_solve": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.POINTER(SolveOpts), C.POINTER(SolveStats)]),
    "pcd_poisson_solve_device": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.POINTER(SolveOpts),
                                           C.POINTER(SolveStats), _vp]),
    "pcd_subtract_average_device": (C.c_int, [_vp, _vp, C.c_int, C.c_int, _vp]),
    "pcd_batch_solve_device": (C.c_int, [_vp, C.POINTER(Instance), C.c_int, C.POINTER(SolveOpts),
                                         C.POINTER(InstanceStats), C.POINTER(BatchStats), _vp]),
    "pcd_ctx_set_autotune": (C.c_int, [_vp, C.c_int]),
    "pcd_ctx_set_wait_limit": (C.c_int, [_vp, C.c_longlong, C.c_int]),
    "pcd_write_solid_obj": (C.c_int, [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_char_p]),
    "pcd_write_grid_svg": (C.c_int, [_dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_char_p, C.c_double]),
    "pcd_write_heightmap_json": (C.c_int, [_dp, C.c_int, C.c_int, C.c_char_p]),
    "pcd_design_save_solid_obj": (C.c_int, [_vp, C.c_int, C.c_char_p]),
    "pcd_design_export_parameterization_svg": (C.c_int, [_vp, C.c_char_p, C.c_double]),
    "pcd_design_export_inverted_transport_map_svg": (C.c_int, [_vp, C.c_char_p, C.c_double]),
    "pcd_design_save_heightmap_json": (C.c_int, [_vp, C.c_char_p]),
    "pcd_design_smooth_target_mesh": (C.c_int, [_vp, C.c_double]),
    "pcd_image_to_grid": (C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp]),
    "pcd_png_decode": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_char_p]),
    "pcd_resize_image": (C.c_int, [_dp, C.c_int, C.c_int, _dp, C.c_int, C.c_int]),
    "pcd_resize_image_device": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    "pcd_design_count_folds": (C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    "pcd_design_set_target_points": (C.c_int, [_vp, _dp]),
    "pcd_ctx_autotune_info": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "pcd_gradient_device": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, _vp]),
    "pcd_divergence_device": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, _vp]),
    "pcd_subtract_average_noalloc": (C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    "pcd_unet_create": (C.c_int, [_vp, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(_vp)]),
    "pcd_unet_destroy": (C.c_int, [_vp]),
    "pcd_unet_num_params": (C.c_longlong, [_vp]),
    "pcd_unet_resolution": (C.c_int, [_vp]),
    "pcd_unet_get_params": (C.c_int, [_vp, _vp]),
    "pcd_unet_set_params": (C.c_int, [_vp, _vp]),
    "pcd_unet_get_grads": (C.c_int, [_vp, _vp]),
    "pcd_unet_train_step": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_float, C.c_float, C.POINTER(C.c_float), _vp]),
    "pcd_unet_predict": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "pcd_ctx_set_warm_start_net": (C.c_int, [_vp, _vp]),
    "pcd_gemm_bf16": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp,
                                _vp]),
    "pcd_gemm_bf16_path": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                     _vp, C.c_int, _vp]),
    "pcd_gemm_bf16_status": (C.c_int, []),
    "pcd_conv3x3_bf16": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, C.c_int, C.c_int, _vp,
                                   C.c_int, _vp]),
    "pcd_conv3x3_wgrad_bf16": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, C.c_int, _vp,
                                         C.c_int, C.c_int, _vp, _vp]),
    "pcd_gemm_bf16_layout": (C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_int, C.c_int, _vp, _vp]),
    "pcd_gemm_set_default_path": (C.c_int, [C.c_int]),
    "pcd_design_params_default": (C.c_int, [C.POINTER(DesignParams)]),
    "pcd_design_create": (C.c_int, [_vp, C.POINTER(DesignParams), C.POINTER(_vp)]),
    "pcd_design_destroy": (C.c_int, [_vp]),
    "pcd_design_initialize": (C.c_int, [_vp, _vp]),
    "pcd_design_transport_iteration": (C.c_int, [_vp, _dp, C.POINTER(SolveStats)]),
    "pcd_design_height_iteration": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(SolveStats)]),
    "pcd_design_initialize_batch": (C.c_int, [_vp, C.c_int, _vp, C.POINTER(C.c_int)]),
    "pcd_design_transport_iteration_batch": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(SolveStats),
                                                       C.POINTER(C.c_int)]),
    "pcd_design_height_iteration_batch": (C.c_int, [_vp, C.c_int, C.c_int, _dp, C.POINTER(SolveStats),
                                                    C.POINTER(C.c_int)]),
    "pcd_design_get_grid": (C.c_int, [_vp, C.c_int, _vp]),
    "pcd_design_get_vertices": (C.c_int, [_vp, C.c_int, _vp]),
}


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) or (build_if_missing and not _build.up_to_date()):
            if not build_if_missing:
                raise RuntimeError(f"libpcd_gb300 not built at {path}")
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def status_string(status: int) -> str:
    try:
        return load(False).pcd_status_string(status).decode()
    except Exception:
        return str(status)


def check(status: int, where: str, ok=(PCD_OK,)) -> int:
    if status in ok:
        return status
    L = load(False)
    raise PCDError(status, where, L.pcd_last_error().decode())


def default_opts() -> SolveOpts:
    o = SolveOpts()
    load().pcd_solve_opts_default(C.byref(o))
    return o
