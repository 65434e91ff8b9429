"""ctypes binding of libtdic_gb300.so (the C ABI in include/tdic_gb300.h).

There is no CPU fallback: if the CUDA library is missing or no GPU is visible, every compute
call raises.  Build the library with ``build.build()`` (nvcc, sm_103a).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtdic_gb300.so")

TDIC_OK, TDIC_INVALID_ARG, TDIC_OOM, TDIC_CUDA_ERROR, TDIC_TIMEOUT, TDIC_UNSUPPORTED = range(6)
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT", 5: "UNSUPPORTED"}
DTYPES = {"uint8": 0, "uint16": 1, "float32": 2, "float64": 3}
HOST, DEVICE = 0, 1
FP32_MIXED, FP64 = 0, 1

CONFIG_FIELDS = [
    ("subset_radius", C.c_int32), ("max_iterations", C.c_int32), ("convergence_threshold", C.c_double),
    ("optimizer", C.c_int32), ("shape_order", C.c_int32), ("criterion", C.c_int32), ("degree", C.c_int32),
    ("border", C.c_int32), ("propagation_spacing", C.c_int32), ("propagation_max_znssd", C.c_double),
    ("is_subset_radius", C.c_int32), ("is_search_radius", C.c_int32), ("sift_enabled", C.c_int32),
    ("pyramid_enabled", C.c_int32), ("pyramid_scale", C.c_int32), ("pyramid_refinement_radius", C.c_int32),
    ("sp_enabled", C.c_int32), ("sp_subset_radius", C.c_int32), ("sp_max_iterations", C.c_int32),
    ("precision", C.c_int32), ("sp_convergence_threshold", C.c_double), ("seed_count", C.c_int32),
    ("kmeans_iterations", C.c_int32), ("seed_max_znssd", C.c_double), ("min_displacement_norm", C.c_double),
    ("min_texture_std", C.c_double), ("kmeans_sample_limit", C.c_int32), ("propagation_mode", C.c_int32),
    ("truncate_roi_subsets", C.c_int32), ("min_valid_samples", C.c_int32), ("min_valid_sample_ratio", C.c_double),
    ("staging", C.c_int32), ("pad_", C.c_int32),
]


class Config(C.Structure):
    _fields_ = CONFIG_FIELDS

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in CONFIG_FIELDS}


class PoiIn(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("p0", C.c_double * 6), ("confidence", C.c_double)]


class PoiOut(C.Structure):
    _fields_ = [("p", C.c_double * 6), ("correlation", C.c_double), ("zncc", C.c_double), ("iterations", C.c_int32),
                ("status", C.c_int8), ("valid", C.c_int8), ("converged", C.c_int8), ("pad_", C.c_int8),
                ("q", C.c_double * 6)]


class Seed(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("p", C.c_double * 6), ("correlation", C.c_double),
                ("found", C.c_int32), ("pad_", C.c_int32)]


GRID_FIELDS = ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "zncc", "valid", "status",
               "iterations", "converged")
# second-order terms of dic::Displacement2D (written for shape_order 2, zero otherwise)
SECOND_ORDER_FIELDS = ("d2u_dx2", "d2u_dxdy", "d2u_dy2", "d2v_dx2", "d2v_dxdy", "d2v_dy2")


class LsStrain(C.Structure):
    _fields_ = [("du_dx", C.c_double), ("du_dy", C.c_double), ("dv_dx", C.c_double), ("dv_dy", C.c_double),
                ("exx", C.c_double), ("eyy", C.c_double), ("exy", C.c_double), ("sample_count", C.c_int32),
                ("valid", C.c_uint8), ("pad_", C.c_uint8 * 3)]


class GridOut(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in GRID_FIELDS + SECOND_ORDER_FIELDS]


# Every exported symbol of include/tdic_gb300.h with its ctypes signature.
SIGNATURES = {
    "tdic_config_default": (None, [C.POINTER(Config)]),
    "tdic_grid_dims": (None, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "tdic_subset_padding": (C.c_int32, [C.POINTER(Config)]),
    "tdic_subset_grid_dims": (None, [C.c_int32, C.c_int32, C.POINTER(Config), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
    "tdic_solve_pois_masked": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Config), C.c_void_p, C.c_void_p,
                                         C.c_int32, C.c_void_p, C.c_int, C.c_void_p]),
    "tdic_ctx_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
    "tdic_ctx_destroy": (None, [C.c_void_p]),
    "tdic_last_error": (C.c_char_p, [C.c_void_p]),
    "tdic_ctx_device_bytes": (C.c_size_t, [C.c_void_p]),
    "tdic_pair_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int,
                                   C.c_int, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                   C.POINTER(C.c_void_p)]),
    "tdic_pair_update": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int, C.c_int, C.c_void_p]),
    "tdic_pair_destroy": (None, [C.c_void_p]),
    "tdic_pair_coefficients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "tdic_pair_images": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "tdic_reference_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "tdic_solve_pois": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Config), C.c_void_p, C.c_int32, C.c_void_p,
                                  C.c_int, C.c_void_p]),
    "tdic_propagate": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Config), C.POINTER(Seed), C.c_void_p,
                                 C.POINTER(GridOut), C.c_int, C.POINTER(C.c_int32), C.c_void_p]),
    "tdic_propagate_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Config), C.POINTER(Seed), C.c_void_p,
                                         C.POINTER(GridOut), C.POINTER(C.c_int32), C.c_void_p]),
    "tdic_batch_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_void_p)]),
    "tdic_batch_tune": (C.c_int, [C.c_void_p, C.c_void_p]),
    "tdic_batch_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "tdic_batch_finish": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "tdic_batch_outputs": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(GridOut)]),
    "tdic_batch_results": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(GridOut), C.c_void_p]),
    "tdic_batch_set_sms": (C.c_int, [C.c_void_p, C.c_int32]),
    "tdic_ctx_heap_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_double)]),
    "tdic_batch_config": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "tdic_batch_destroy": (None, [C.c_void_p]),
    "tdic_subset_prepare": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_void_p,
                                      C.POINTER(Config), C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(Seed)]),
    "tdic_write_subset_csv": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_int, C.c_int32]),
    "tdic_ls_strain_2d": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                    C.c_void_p, C.c_void_p]),
    "tdic_select_seed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Config),
                                   C.POINTER(Seed), C.c_void_p]),
    "tdic_integer_search": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Config), C.c_void_p, C.c_void_p, C.c_int32,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tdic_subset_compute": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_void_p,
                                      C.POINTER(Config), C.POINTER(GridOut), C.POINTER(C.c_int32), C.POINTER(Seed),
                                      C.c_void_p]),
}

_lock = threading.Lock()
_lib = None


class TdicError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(path: str | None = None):
    """Load the CUDA library (building it first if it is absent).  Raises when it cannot."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            from . import build as _build
            _build.build()
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def default_config() -> Config:
    cfg = Config()
    load().tdic_config_default(C.byref(cfg))
    return cfg


def grid_dims(w: int, h: int, spacing: int):
    gw, gh = C.c_int32(), C.c_int32()
    load().tdic_grid_dims(w, h, spacing, C.byref(gw), C.byref(gh))
    return gw.value, gh.value


def subset_grid_dims(w: int, h: int, cfg: Config):
    """Output grid of tdic_subset_compute (with truncate_roi_subsets: the padded grid cropped to the image)."""
    gw, gh = C.c_int32(), C.c_int32()
    load().tdic_subset_grid_dims(w, h, C.byref(cfg), C.byref(gw), C.byref(gh))
    return gw.value, gh.value


def check(status: int, ctx) -> None:
    if status != TDIC_OK:
        msg = load().tdic_last_error(ctx).decode()  # NULL: this thread's context-free message
        raise TdicError(status, msg)
