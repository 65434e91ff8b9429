"""ctypes wrapper of the FP64 CPU oracle (oracle/tdic_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the checker and by
bench.py's CPU-baseline leg.  The product never imports this module.

The C library restates the reference's hot path (lbd-hfut/Traditional-DIC): B-spline
prefilter (src/interpolation/bspline.cpp:369-392), reference gradient cache
(src/subset/seed/reliability_propagation.cpp:84-112), first-order ZNSSD ICGN
(src/subset/solver/icgn.cpp:446-627), first-order FGN
(src/subset/solver/forward_gauss_newton.cpp:188-399), their SSD and second-order variants
(icgn.cpp:832-988, 1168-1362, 1576-1739; forward_gauss_newton.cpp:622-794, 1069-1297, 1540-1739),
reliability-guided propagation
(reliability_propagation.cpp:130-394), integer search (src/initialization/integer_search.cpp:333-432)
and seed selection (src/subset/seed/seed_selector.cpp:146-317).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libtdic_oracle.so")
_lock = threading.Lock()
_lib = None

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


class PoiResult(C.Structure):
    _fields_ = [("p", C.c_double * 6), ("correlation", C.c_double), ("iterations", C.c_int32),
                ("status", C.c_int8), ("valid", C.c_int8), ("converged", C.c_int8), ("pad_", C.c_int8),
                ("q", C.c_double * 6)]


SECOND_ORDER_KEYS = ("d2u_dx2", "d2u_dxdy", "d2u_dy2", "d2v_dx2", "d2v_dxdy", "d2v_dy2")


class GridOut(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy",
                                           "correlation", "valid", "status", "iterations", "converged")
                + SECOND_ORDER_KEYS]


class Seed(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("p", C.c_double * 6), ("correlation", C.c_double),
                ("found", C.c_int32), ("pad_", C.c_int32)]


GRID_KEYS = ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation")


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (portable flags; runs on x86_64 and aarch64)."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "tdic_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            P = C.c_void_p
            L.orc_config_default.argtypes = [C.POINTER(Config)]
            L.orc_bspline_basis.restype = C.c_double
            L.orc_bspline_basis.argtypes = [C.c_double, C.c_int, C.c_int]
            L.orc_bspline_qk.argtypes = [C.c_int, P]
            L.orc_prefilter.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P]
            L.orc_interp_value.restype = C.c_double
            L.orc_interp_value.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
            L.orc_interp_gradient.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, P, P]
            L.orc_reference_gradient.argtypes = [P, C.c_int, C.c_int, P, P]
            L.orc_solve_pois.argtypes = [P, C.c_int, C.c_int, P, P, P, C.c_int, C.c_int, C.POINTER(Config),
                                         C.c_int, P, P, P, P]
            L.orc_solve_pois_masked.argtypes = [P, C.c_int, C.c_int, P, P, P, P, C.c_int, C.c_int, C.POINTER(Config),
                                                C.c_int, P, P, P, P]
            L.orc_grid_dims.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
            L.orc_subset_padding.argtypes = [C.POINTER(Config)]
            L.orc_truncated_grid_dims.argtypes = [C.c_int, C.c_int, C.POINTER(Config), C.POINTER(C.c_int),
                                                  C.POINTER(C.c_int)]
            L.orc_propagate.argtypes = [P, C.c_int, C.c_int, P, P, P, P, C.POINTER(Config), C.POINTER(Seed),
                                        C.c_int, C.POINTER(GridOut), C.POINTER(C.c_int)]
            L.orc_propagate_threads.argtypes = [P, C.c_int, C.c_int, P, P, P, P, C.POINTER(Config),
                                                C.POINTER(Seed), C.c_int, C.POINTER(GridOut), C.POINTER(C.c_int),
                                                C.c_int]
            L.orc_integer_search.argtypes = [P, P, C.c_int, C.c_int, C.POINTER(Config), C.c_double, C.c_double,
                                             C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.orc_integer_search_masked.argtypes = [P, P, C.c_int, C.c_int, P, C.POINTER(Config), C.c_double,
                                                    C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                    C.POINTER(C.c_double)]
            L.orc_select_seed.argtypes = [P, P, C.c_int, C.c_int, P, C.POINTER(Config), C.POINTER(Seed), P,
                                          C.c_int, C.POINTER(C.c_int)]
            L.orc_subset_compute.argtypes = [P, P, C.c_int, C.c_int, P, C.POINTER(Config), C.POINTER(GridOut),
                                             C.POINTER(Seed)]
            _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def default_config(**overrides) -> Config:
    cfg = Config()
    lib().orc_config_default(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def as_config(cfg) -> Config:
    """Accept an oracle Config, a byte-compatible structure (the product's tdic_config) or a dict."""
    if cfg is None:
        return default_config()
    if isinstance(cfg, Config):
        return cfg
    if isinstance(cfg, dict):
        return default_config(**cfg)
    out = Config()
    C.memmove(C.byref(out), C.byref(cfg), C.sizeof(Config))
    return out


def _img(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def basis(x: float, r: int, degree: int) -> float:
    return lib().orc_bspline_basis(float(x), int(r), int(degree))


def qk(degree: int) -> np.ndarray:
    out = np.zeros((degree + 1, degree + 1), np.float64)
    if lib().orc_bspline_qk(degree, _ptr(out)) != 0:
        raise ValueError("degree must be 1, 3 or 5")
    return out


def prefilter(image, degree: int = 3, border: int = 3, exact: bool = True) -> np.ndarray:
    img = _img(image)
    h, w = img.shape
    b = max(3, border)
    out = np.zeros((h + 2 * b, w + 2 * b), np.float64)
    if lib().orc_prefilter(_ptr(img), w, h, degree, border, int(exact), _ptr(out)) != 0:
        raise ValueError("bad prefilter arguments")
    return out


def interp_value(coeffs, w, h, degree, border, x, y) -> float:
    c = np.ascontiguousarray(coeffs, np.float64)
    return lib().orc_interp_value(_ptr(c), w, h, degree, border, float(x), float(y))


def interp_gradient(coeffs, w, h, degree, border, x, y):
    c = np.ascontiguousarray(coeffs, np.float64)
    gx, gy = C.c_double(), C.c_double()
    lib().orc_interp_gradient(_ptr(c), w, h, degree, border, float(x), float(y), C.addressof(gx), C.addressof(gy))
    return gx.value, gy.value


def reference_gradient(image):
    img = _img(image)
    h, w = img.shape
    gx = np.zeros((h, w), np.float64)
    gy = np.zeros((h, w), np.float64)
    lib().orc_reference_gradient(_ptr(img), w, h, _ptr(gx), _ptr(gy))
    return gx, gy


def solve_pois(reference, coeffs, cfg, xy, p0, confidence0=None, gradients=None, degree=None, border=None,
               roi=None, masked=False):
    """Per-POI solve: ICGN or FGN (cfg.optimizer), first or second order (cfg.shape_order), ZNSSD or
    SSD (cfg.criterion 1 / 0).  Returns a dict of arrays; "q" holds the six second-order terms."""
    cfg = as_config(cfg)
    ref = _img(reference)
    h, w = ref.shape
    xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
    p0 = np.ascontiguousarray(p0, np.float64).reshape(-1, 6)
    n = xy.shape[0]
    conf = None if confidence0 is None else np.ascontiguousarray(confidence0, np.float64)
    gx = gy = None
    if gradients is not None:
        gx = np.ascontiguousarray(gradients[0], np.float64)
        gy = np.ascontiguousarray(gradients[1], np.float64)
    c = np.ascontiguousarray(coeffs, np.float64)
    out = (PoiResult * max(n, 1))()
    d = cfg.degree if degree is None else degree
    b = cfg.border if border is None else border
    if masked:  # solve_with_mask over roi (None: every pixel valid)
        m = None if roi is None else np.ascontiguousarray(roi != 0, np.uint8)
        rc = lib().orc_solve_pois_masked(_ptr(ref), w, h, _ptr(m), _ptr(gx), _ptr(gy), _ptr(c), d, b, C.byref(cfg),
                                         n, _ptr(xy), _ptr(p0), _ptr(conf), C.addressof(out))
    else:
        rc = lib().orc_solve_pois(_ptr(ref), w, h, _ptr(gx), _ptr(gy), _ptr(c), d, b, C.byref(cfg), n,
                                  _ptr(xy), _ptr(p0), _ptr(conf), C.addressof(out))
    if rc != 0:
        raise ValueError("degree must be 1, 3 or 5")
    arr = np.frombuffer(out, dtype=np.dtype([("p", "<f8", 6), ("correlation", "<f8"), ("iterations", "<i4"),
                                              ("status", "i1"), ("valid", "i1"), ("converged", "i1"),
                                              ("pad", "i1"), ("q", "<f8", 6)]), count=n)
    return {"p": arr["p"].copy(), "q": arr["q"].copy(), "correlation": arr["correlation"].copy(),
            "iterations": arr["iterations"].copy(), "status": arr["status"].copy(),
            "valid": arr["valid"].astype(bool), "converged": arr["converged"].astype(bool)}


def subset_padding(cfg) -> int:
    """recommended_subset_padding (src/subset/padding.cpp:28-36)."""
    return lib().orc_subset_padding(C.byref(as_config(cfg)))


def truncated_grid_dims(w, h, cfg):
    """Grid of subset_compute's output when truncating (the padded grid cropped to the image)."""
    gw, gh = C.c_int(), C.c_int()
    lib().orc_truncated_grid_dims(w, h, C.byref(as_config(cfg)), C.byref(gw), C.byref(gh))
    return gw.value, gh.value


def grid_dims(w, h, spacing):
    gw, gh = C.c_int(), C.c_int()
    lib().orc_grid_dims(w, h, spacing, C.byref(gw), C.byref(gh))
    return gw.value, gh.value


def _alloc_grid(n):
    arrs = {k: np.zeros(n, np.float64) for k in GRID_KEYS + SECOND_ORDER_KEYS}
    arrs["valid"] = np.zeros(n, np.uint8)
    arrs["status"] = np.zeros(n, np.int8)
    arrs["iterations"] = np.zeros(n, np.int32)
    arrs["converged"] = np.zeros(n, np.uint8)
    g = GridOut(**{k: arrs[k].ctypes.data for k in arrs})
    return arrs, g


def _finish_grid(arrs, n):
    out = {k: arrs[k][:n] for k in GRID_KEYS + SECOND_ORDER_KEYS}
    out["valid"] = arrs["valid"][:n].astype(bool)
    out["zncc"] = np.clip(1.0 - 0.5 * out["correlation"], -1.0, 1.0)
    out["iterations"] = arrs["iterations"][:n]
    out["converged"] = arrs["converged"][:n].astype(bool)
    out["status"] = arrs["status"][:n]
    return out


def make_seed(x, y, p, correlation) -> Seed:
    s = Seed()
    s.x, s.y = float(x), float(y)
    for i in range(6):
        s.p[i] = float(p[i])
    s.correlation = float(correlation)
    s.found = 1
    return s


def propagate(reference, deformed_coeffs, cfg, seed: Seed, roi=None, gradients=None, max_solves: int = -1,
              threads: int = 1):
    """ReliabilityPropagation::propagate with one seed.  ``threads`` > 1 solves each frontier wave
    (propagation_mode 0) or dataflow diagonal (mode 2) on that many host threads; the result is
    the same for every thread count, and the heap order (mode 1) is always serial."""
    cfg = as_config(cfg)
    ref = _img(reference)
    h, w = ref.shape
    if gradients is None:
        gradients = reference_gradient(ref)
    gx = np.ascontiguousarray(gradients[0], np.float64)
    gy = np.ascontiguousarray(gradients[1], np.float64)
    c = np.ascontiguousarray(deformed_coeffs, np.float64)
    r = None if roi is None else np.ascontiguousarray(roi != 0, np.uint8)
    gw, gh = grid_dims(w, h, cfg.propagation_spacing)
    arrs, g = _alloc_grid(gw * gh)
    solves = C.c_int()
    computed = lib().orc_propagate_threads(_ptr(ref), w, h, _ptr(r), _ptr(gx), _ptr(gy), _ptr(c), C.byref(cfg),
                                           C.byref(seed), int(max_solves), C.byref(g), C.byref(solves),
                                           max(1, int(threads)))
    out = _finish_grid(arrs, gw * gh)
    out["points_computed"] = computed
    out["solves"] = solves.value
    out["grid_shape"] = (gh, gw)
    return out


def integer_search(reference, deformed, cfg, x, y, roi=None):
    """IntegerSearchInitializer::estimate at (x, y); with ``roi`` the masked search.  Returns
    (u, v, zncc) or None."""
    cfg = as_config(cfg)
    ref, de = _img(reference), _img(deformed)
    h, w = ref.shape
    u, v, z = C.c_double(), C.c_double(), C.c_double()
    if roi is None:
        ok = lib().orc_integer_search(_ptr(ref), _ptr(de), w, h, C.byref(cfg), float(x), float(y),
                                      C.byref(u), C.byref(v), C.byref(z))
    else:
        r = np.ascontiguousarray(roi != 0, np.uint8)
        ok = lib().orc_integer_search_masked(_ptr(ref), _ptr(de), w, h, _ptr(r), C.byref(cfg), float(x), float(y),
                                             C.byref(u), C.byref(v), C.byref(z))
    return (u.value, v.value, z.value) if ok else None


def select_seed(reference, deformed, cfg, roi=None):
    cfg = as_config(cfg)
    ref, de = _img(reference), _img(deformed)
    h, w = ref.shape
    r = None if roi is None else np.ascontiguousarray(roi != 0, np.uint8)
    seed = Seed()
    cap = max(1, int(cfg.seed_count))
    cand = np.zeros((cap, 2), np.float64)
    n = C.c_int()
    lib().orc_select_seed(_ptr(ref), _ptr(de), w, h, _ptr(r), C.byref(cfg), C.byref(seed), _ptr(cand), cap,
                          C.byref(n))
    return seed, cand[:min(n.value, cap)].copy()


def subset_compute(reference, deformed, cfg=None, roi=None):
    """Full reference pipeline (SubsetDIC::compute, subset_dic.cpp:39-105); returns the result dict."""
    cfg = as_config(cfg)
    ref, de = _img(reference), _img(deformed)
    h, w = ref.shape
    r = None if roi is None else np.ascontiguousarray(roi != 0, np.uint8)
    pad = subset_padding(cfg) if cfg.truncate_roi_subsets else 0
    gw, gh = grid_dims(w + 2 * pad, h + 2 * pad, cfg.propagation_spacing)
    arrs, g = _alloc_grid(gw * gh)
    seed = Seed()
    n = lib().orc_subset_compute(_ptr(ref), _ptr(de), w, h, _ptr(r), C.byref(cfg), C.byref(g), C.byref(seed))
    out = _finish_grid(arrs, n)
    out["seed"] = seed
    return out
