"""Host-side mirror of the reference's subset-DIC interface over the GB300 C ABI.

``compute(reference, deformed, config=None, roi=None)`` mirrors the pybind entry
``_traditional_dic.subset.compute`` (bindings/python/bind_subset.cpp:253-356) -- argument
checks, config dict parsing (``config_from_dict``, bind_subset.cpp:158-248) and the result dict
of ``results_to_dict`` (bind_subset.cpp:102-153) -- and ``subset(...)`` mirrors the Python API
``traditional_dic.subset`` (python/traditional_dic/subset.py:16-160) with its keyword defaults.
Both run on the GPU through libtdic_gb300.so; there is no CPU fallback.

Additive result keys (not in the reference): ``zncc`` = clamp(1 - correlation / 2),
``iterations``, ``converged`` (strict |dp| < threshold) and ``status`` (dic::SolverStatus).
GPU-only settings live under a separate ``"gpu"`` section of the config dict, which the
reference parser ignores: ``{"gpu": {"precision": "fp32" | "fp64", "propagation": "dataflow" | "waves",
"staging": "auto" | "full" | "lean" | "lean_no_window"}}`` (staging changes speed and shared-memory
needs, never a result).
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from typing import Any

import numpy as np

from . import _lib as L

RESULT_KEYS = ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "valid")
# Visit orders of the propagation: the reference's heap order (reproduced exactly on the device
# in rounds), frontier waves, dataflow (the default)
PROPAGATION_MODES = {"waves": 0, "heap": 1, "dataflow": 2}
EXTRA_KEYS = ("zncc", "iterations", "converged", "status")
# shared-memory staging of the first-order ZNSSD solves (tdic_staging); "gpu": {"staging": ...}
STAGING = {"auto": 0, "full": 1, "lean": 2, "lean_no_window": 3}
STAGING_NAMES = {v: k for k, v in STAGING.items()}


# ---------------------------------------------------------------------------------------------
# Context / pair handles
# ---------------------------------------------------------------------------------------------
class Context:
    """One device, one stream, a caching device-memory pool (tdic_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        st = self.lib.tdic_ctx_create(int(device), C.byref(h))
        if st != L.TDIC_OK:
            why = self.lib.tdic_last_error(None).decode()
            raise L.TdicError(st, f"cannot create a context on device {device}: {why}")
        self.handle = h
        self.device = device

    def check(self, status: int) -> None:
        L.check(status, self.handle)

    @property
    def device_bytes(self) -> int:
        return int(self.lib.tdic_ctx_device_bytes(self.handle))

    def heap_stats(self) -> tuple:
        """(device rounds, solves in them, host ms in the heap simulations) of the last
        heap-order propagation on this context."""
        r, n, ms = C.c_int32(), C.c_int64(), C.c_double()
        self.check(self.lib.tdic_ctx_heap_stats(self.handle, C.byref(r), C.byref(n), C.byref(ms)))
        return r.value, n.value, ms.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.tdic_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_lock = threading.Lock()
_default_ctx: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    with _default_lock:
        ctx = _default_ctx.get(device)
        if ctx is None:
            ctx = Context(device)
            _default_ctx[device] = ctx
        return ctx


def _image_arg(a) -> tuple[int, int, int, int, int, Any]:
    """(pointer, width, height, dtype code, memory, keepalive) for a numpy array or CUDA tensor."""
    if hasattr(a, "data_ptr") and getattr(a, "is_cuda", False):
        if a.dim() != 2:
            raise RuntimeError("Image must be a 2D numpy array.")
        if not a.is_contiguous():
            a = a.contiguous()
        name = str(a.dtype).replace("torch.", "")
        if name not in L.DTYPES:
            raise TypeError(f"unsupported image dtype {name}")
        return a.data_ptr(), int(a.shape[1]), int(a.shape[0]), L.DTYPES[name], L.DEVICE, a
    arr = np.asarray(a)
    if arr.ndim != 2:
        raise RuntimeError("Image must be a 2D numpy array.")
    if arr.dtype.name not in L.DTYPES:
        raise RuntimeError("reference must be a 2D numpy array (float32 or float64).")
    arr = np.ascontiguousarray(arr)
    return arr.ctypes.data, int(arr.shape[1]), int(arr.shape[0]), L.DTYPES[arr.dtype.name], L.HOST, arr


class Pair:
    """A reference / deformed image pair resident on the device (tdic_pair): the float32
    reference and the deformed image's B-spline coefficients (BSplineImagePreprocessor::compute,
    src/interpolation/bspline.cpp:270-300)."""

    def __init__(self, ctx: Context, reference, deformed, degree: int = 3, border: int = 3, exact: bool = True,
                 precision: int = L.FP32_MIXED, stream=None):
        self.ctx = ctx
        rp, w, h, dt, mem, self._keep_r = _image_arg(reference)
        dp, w2, h2, dt2, mem2, self._keep_d = _image_arg(deformed)
        if (w, h, dt, mem) != (w2, h2, dt2, mem2):
            raise ValueError("reference and deformed must have the same shape, dtype and memory")
        self.width, self.height, self.degree, self.precision = w, h, degree, precision
        self.border = max(3, border)
        hnd = C.c_void_p()
        ctx.check(ctx.lib.tdic_pair_create(ctx.handle, rp, dp, w, h, 0, dt, mem, degree, border, int(exact), precision,
                                           _stream_ptr(stream), C.byref(hnd)))
        self.handle = hnd

    @classmethod
    def _adopt(cls, ctx: Context, handle: C.c_void_p, width: int, height: int, degree: int, precision: int,
               border: int) -> "Pair":
        """Wrap a pair the library created (tdic_subset_prepare)."""
        self = cls.__new__(cls)
        self.ctx, self.handle = ctx, handle
        self.width, self.height, self.degree, self.precision = width, height, degree, precision
        self.border = max(3, border)
        return self

    def update(self, reference, deformed, stream=None) -> None:
        """New images for the pair: the pair's shape; both of one dtype and memory kind (the
        library reads the two buffers with the one dtype it is given)."""
        rp, w, h, dt, mem, keep_r = _image_arg(reference)
        dp, w2, h2, dt2, mem2, keep_d = _image_arg(deformed)
        if (w, h) != (self.width, self.height) or (w2, h2) != (self.width, self.height):
            raise ValueError("update needs images of the pair's shape")
        if (dt, mem) != (dt2, mem2):
            raise ValueError("reference and deformed must have the same dtype and memory")
        self._keep_r, self._keep_d = keep_r, keep_d
        self.ctx.check(self.ctx.lib.tdic_pair_update(self.handle, rp, dp, 0, dt, mem, _stream_ptr(stream)))

    def coefficients(self) -> np.ndarray:
        dtype = np.float64 if self.precision == L.FP64 else np.float32
        out = np.empty((self.height + 2 * self.border, self.width + 2 * self.border), dtype)
        self.ctx.check(self.ctx.lib.tdic_pair_coefficients(self.handle, out.ctypes.data, out.nbytes))
        return out

    def images(self) -> tuple:
        """The float32 reference and deformed images the pair holds."""
        r = np.empty((self.height, self.width), np.float32)
        d = np.empty_like(r)
        self.ctx.check(self.ctx.lib.tdic_pair_images(self.handle, r.ctypes.data, d.ctypes.data))
        return r, d

    def reference_gradient(self):
        gx = np.empty((self.height, self.width), np.float64)
        gy = np.empty_like(gx)
        self.ctx.check(self.ctx.lib.tdic_reference_gradient(self.handle, gx.ctypes.data, gy.ctypes.data))
        return gx, gy

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.tdic_pair_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


# ---------------------------------------------------------------------------------------------
# Config parsing: bind_subset.cpp:158-248 (config_from_dict) over the C++ defaults.
# ---------------------------------------------------------------------------------------------
def _gi(d: dict, k: str, default: int) -> int:
    if k not in d:
        return default
    v = d[k]
    if isinstance(v, (bool, np.bool_)):
        return int(v)
    if isinstance(v, (int, np.integer)):
        return int(v)
    raise RuntimeError(f"Unable to cast Python instance of type {type(v)} to C++ type 'int'")


def _gd(d: dict, k: str, default: float) -> float:
    if k not in d:
        return default
    v = d[k]
    if isinstance(v, (int, float, np.integer, np.floating)) and not isinstance(v, str):
        return float(v)
    raise RuntimeError(f"Unable to cast Python instance of type {type(v)} to C++ type 'double'")


def _gb(d: dict, k: str) -> bool:
    v = d[k]
    if isinstance(v, (bool, np.bool_)):
        return bool(v)
    raise RuntimeError(f"Unable to cast Python instance of type {type(v)} to C++ type 'bool'")


def config_from_dict(d: dict | None) -> L.Config:
    cfg = L.default_config()
    if not d:
        return cfg
    if "subset" in d:
        cfg.subset_radius = _gi(d["subset"], "radius", cfg.subset_radius)
    if "optimization" in d:
        o = d["optimization"]
        cfg.max_iterations = _gi(o, "max_iterations", cfg.max_iterations)
        cfg.convergence_threshold = _gd(o, "convergence_threshold", cfg.convergence_threshold)
        if "method" in o:
            m = str(o["method"])
            if m == "icgn":
                cfg.optimizer = 0
            elif m in ("forward_gauss_newton", "fgn"):
                cfg.optimizer = 1
            else:
                raise RuntimeError("subset optimization.method must be 'icgn', 'fgn', or 'forward_gauss_newton'.")
    if "correlation" in d:
        o = d["correlation"]
        if "criterion" in o:
            c = str(o["criterion"])
            if c == "ssd":
                cfg.criterion = 0
            elif c == "znssd":
                cfg.criterion = 1
            else:
                raise RuntimeError("subset correlation.criterion must be 'ssd' or 'znssd'.")
    if "interpolation" in d:
        o = d["interpolation"]
        if "degree" in o:
            deg = _gi(o, "degree", 5)
            if deg in (1, 3):  # any other value leaves the quintic default (bind_subset.cpp:195-200)
                cfg.degree = deg
    if "initialization" in d:
        o = d["initialization"]
        if "method" in o:
            if not isinstance(o["method"], str):
                raise RuntimeError("Unable to cast initialization.method to std::string")
            if o["method"] != "integer_search":
                raise RuntimeError("subset initialization.method must be integer_search")
        if "integer_search" in o:
            s = o["integer_search"]
            cfg.is_subset_radius = _gi(s, "subset_radius", cfg.is_subset_radius)
            cfg.is_search_radius = _gi(s, "search_radius", cfg.is_search_radius)
            if "sift_enabled" in s:
                cfg.sift_enabled = int(_gb(s, "sift_enabled"))
            if "pyramid_enabled" in s:
                cfg.pyramid_enabled = int(_gb(s, "pyramid_enabled"))
            cfg.pyramid_scale = _gi(s, "pyramid_scale", cfg.pyramid_scale)
            cfg.pyramid_refinement_radius = _gi(s, "pyramid_refinement_radius", cfg.pyramid_refinement_radius)
        if "subpixel_refinement" in o:
            s = o["subpixel_refinement"]
            if "enabled" in s:
                cfg.sp_enabled = int(_gb(s, "enabled"))
            cfg.sp_subset_radius = _gi(s, "subset_radius", cfg.sp_subset_radius)
            cfg.sp_max_iterations = _gi(s, "max_iterations", cfg.sp_max_iterations)
            cfg.sp_convergence_threshold = _gd(s, "convergence_threshold", cfg.sp_convergence_threshold)
    if "seed_selection" in d:
        o = d["seed_selection"]
        cfg.seed_count = _gi(o, "seed_count", cfg.seed_count)
        cfg.seed_max_znssd = _gd(o, "max_znssd", cfg.seed_max_znssd)
        cfg.min_displacement_norm = _gd(o, "min_displacement_norm", cfg.min_displacement_norm)
        cfg.min_texture_std = _gd(o, "min_texture_std", cfg.min_texture_std)
        cfg.kmeans_iterations = _gi(o, "kmeans_iterations", cfg.kmeans_iterations)
        cfg.kmeans_sample_limit = _gi(o, "kmeans_sample_limit", cfg.kmeans_sample_limit)
    if "reliability_propagation" in d:
        o = d["reliability_propagation"]
        cfg.propagation_spacing = _gi(o, "spacing", cfg.propagation_spacing)
        cfg.propagation_max_znssd = _gd(o, "max_znssd", cfg.propagation_max_znssd)
    if "shape_function" in d:
        s = d["shape_function"]
        if "order" in s:
            order = str(s["order"])
            if order in ("first_order", "1"):
                cfg.shape_order = 1
            elif order in ("second_order", "2"):
                cfg.shape_order = 2
            else:
                raise RuntimeError("subset shape_function.order must be 'first_order'/'1' or 'second_order'/'2'.")
    gpu = d.get("gpu") or {}
    if "precision" in gpu:
        p = str(gpu["precision"]).lower()
        if p not in ("fp32", "fp64"):
            raise RuntimeError("gpu.precision must be 'fp32' or 'fp64'.")
        cfg.precision = L.FP64 if p == "fp64" else L.FP32_MIXED
    if "propagation" in gpu:
        m = str(gpu["propagation"]).lower()
        if m not in PROPAGATION_MODES:
            raise RuntimeError("gpu.propagation must be 'heap', 'waves' or 'dataflow'.")
        cfg.propagation_mode = PROPAGATION_MODES[m]
    if "staging" in gpu:
        m = str(gpu["staging"]).lower()
        if m not in STAGING:
            raise RuntimeError("gpu.staging must be 'auto', 'full', 'lean' or 'lean_no_window'.")
        cfg.staging = STAGING[m]
    return cfg


# ---------------------------------------------------------------------------------------------
# Result dicts
# ---------------------------------------------------------------------------------------------
def _empty_result() -> dict:
    out = {k: np.zeros(0, np.float64) for k in RESULT_KEYS}
    out["valid"] = np.zeros(0, bool)
    out["zncc"] = np.zeros(0, np.float64)
    out["iterations"] = np.zeros(0, np.int32)
    out["converged"] = np.zeros(0, bool)
    out["status"] = np.zeros(0, np.int8)
    return out


def _alloc_grid(n: int, second_order: bool = False):
    arrs = {k: np.zeros(n, np.float64) for k in ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation",
                                                  "zncc")}
    arrs["valid"] = np.zeros(n, np.uint8)
    arrs["status"] = np.zeros(n, np.int8)
    arrs["iterations"] = np.zeros(n, np.int32)
    arrs["converged"] = np.zeros(n, np.uint8)
    keys = L.GRID_FIELDS
    if second_order:
        for k in L.SECOND_ORDER_FIELDS:
            arrs[k] = np.zeros(n, np.float64)
        keys = keys + L.SECOND_ORDER_FIELDS
    g = L.GridOut(**{k: arrs[k].ctypes.data for k in keys})
    return arrs, g


def _finish(arrs: dict) -> dict:
    """The reference's result dict (results_to_dict, bind_subset.cpp:102-153) plus the additive
    keys; for the second-order shape function also the six second-order terms."""
    out = {k: arrs[k] for k in RESULT_KEYS if k != "valid"}
    out["valid"] = arrs["valid"].astype(bool)
    out["zncc"] = arrs["zncc"]
    out["iterations"] = arrs["iterations"]
    out["converged"] = arrs["converged"].astype(bool)
    out["status"] = arrs["status"]
    res = {k: out[k] for k in RESULT_KEYS + EXTRA_KEYS}
    for k in L.SECOND_ORDER_FIELDS:
        if k in arrs:
            res[k] = arrs[k]
    return res


def _roi_arg(roi, w: int, h: int):
    if roi is None:
        return None, None
    r = np.asarray(roi)
    if r.dtype not in (np.bool_, np.uint8):
        raise RuntimeError("roi must be a 2D numpy array (bool or uint8) or None.")
    if r.ndim != 2:
        raise RuntimeError("Mask must be a 2D numpy array.")
    if r.shape != (h, w):
        return "mismatch", None
    r = np.ascontiguousarray(r != 0, dtype=np.uint8)
    return r.ctypes.data, r


# ---------------------------------------------------------------------------------------------
# Entry points
# ---------------------------------------------------------------------------------------------
def compute(reference, deformed, config: dict | None = None, roi=None, *, context: Context | None = None,
            return_seed: bool = False):
    """Drop-in for ``_traditional_dic.subset.compute`` (bind_subset.cpp:253-315)."""
    ref = _check_image(reference, "reference")
    de = _check_image(deformed, "deformed")
    if config is not None and not isinstance(config, dict):
        raise RuntimeError("config must be a dict (from YAML) or None.")
    return compute_config(ref, de, config_from_dict(config), roi, context=context, return_seed=return_seed)


def compute_config(reference, deformed, cfg: L.Config, roi=None, *, context: Context | None = None,
                   return_seed: bool = False):
    """``SubsetDIC::compute`` (subset_dic.cpp:39-105) with a full configuration structure: the
    C++ ``SubsetConfig`` knobs the pybind dict does not reach, e.g. ``truncate_roi_subsets`` with
    ``min_valid_samples`` / ``min_valid_sample_ratio`` (masked subsets over padded images; the
    grid points are then gx * step - pad, see ``tdic_subset_grid_dims``)."""
    ref = _check_image(reference, "reference")
    de = _check_image(deformed, "deformed")
    ctx = context or default_context()
    seed = L.Seed()
    if ref.shape != de.shape or ref.size == 0:
        return (_empty_result(), seed) if return_seed else _empty_result()   # SubsetDIC::compute: empty result
    h, w = ref.shape
    rptr, rkeep = _roi_arg(roi, w, h)
    if rptr == "mismatch":
        return (_empty_result(), seed) if return_seed else _empty_result()
    if de.dtype != ref.dtype:
        de = de.astype(ref.dtype)
    gw, gh = L.subset_grid_dims(w, h, cfg)
    arrs, g = _alloc_grid(gw * gh, cfg.shape_order == 2)
    n = C.c_int32()
    ctx.check(ctx.lib.tdic_subset_compute(ctx.handle, ref.ctypes.data, de.ctypes.data, w, h, L.DTYPES[ref.dtype.name],
                                          rptr, C.byref(cfg), C.byref(g), C.byref(n), C.byref(seed), None))
    res = _empty_result() if n.value == 0 else {k: v[:n.value] for k, v in _finish(arrs).items()}
    return (res, seed) if return_seed else res


def _check_image(a, name: str) -> np.ndarray:
    arr = a
    if not isinstance(arr, np.ndarray):
        raise RuntimeError(f"{name} must be a 2D numpy array (float32 or float64).")
    if arr.dtype.name not in ("float32", "float64", "uint8", "uint16"):
        raise RuntimeError(f"{name} must be a 2D numpy array (float32 or float64).")
    if arr.ndim != 2:
        raise RuntimeError("Image must be a 2D numpy array.")
    return np.ascontiguousarray(arr)


def subset(reference: np.ndarray, deformed: np.ndarray, config: str | Path | dict | None = None, roi=None,
           radius: int = 15, max_iterations: int = 30, convergence_threshold: float = 1e-3, bspline_degree: int = 5,
           search_radius: int = 20, seed_subset_radius: int = 10, sift_enabled: bool = False,
           pyramid_enabled: bool = True, subpixel_refinement: bool = True, seed_count: int = 64,
           max_znssd: float = 0.3, min_displacement_norm: float = 0.0, min_texture_std: float = 0.02,
           propagation_spacing: int = 5, propagation_max_znssd: float = 0.5, gpu: dict | None = None):
    """Drop-in for ``traditional_dic.subset`` (python/traditional_dic/subset.py:16-160)."""
    if not isinstance(reference, np.ndarray) or reference.ndim != 2:
        raise ValueError("reference must be a 2D numpy array")
    if not isinstance(deformed, np.ndarray) or deformed.ndim != 2:
        raise ValueError("deformed must be a 2D numpy array")
    if reference.shape != deformed.shape:
        raise ValueError("reference and deformed must have the same shape")
    if config is not None:
        if isinstance(config, (str, Path)):
            raise TypeError("YAML config files need PyYAML, which this package does not depend on; pass a dict")
        if not isinstance(config, dict):
            raise TypeError(f"config must be str, Path, dict, or None, got {type(config)}")
        config_dict = dict(config)
    else:
        config_dict = {
            "subset": {"radius": radius},
            "optimization": {"max_iterations": max_iterations, "convergence_threshold": convergence_threshold},
            "interpolation": {"degree": bspline_degree},
            "initialization": {
                "method": "integer_search",
                "integer_search": {"subset_radius": seed_subset_radius, "search_radius": search_radius,
                                   "sift_enabled": sift_enabled, "pyramid_enabled": pyramid_enabled},
                "subpixel_refinement": {"enabled": subpixel_refinement, "subset_radius": radius,
                                        "max_iterations": max_iterations,
                                        "convergence_threshold": convergence_threshold},
            },
            "seed_selection": {"seed_count": seed_count, "max_znssd": max_znssd,
                               "min_displacement_norm": min_displacement_norm, "min_texture_std": min_texture_std},
            "reliability_propagation": {"spacing": propagation_spacing, "max_znssd": propagation_max_znssd},
        }
    if gpu:
        config_dict["gpu"] = gpu
    return compute(reference, deformed, config_dict, roi)


def solve_pois(ctx: Context, pair: Pair, config: L.Config, xy, p0, confidence=None, roi=None,
               masked: bool = False) -> dict:
    """Batched per-POI solve (tdic_solve_pois) on host arrays, on the config's route (optimizer,
    shape_order, criterion); "q" holds the six second-order terms (zero for first order).
    ``masked``: solve_with_mask over ``roi`` (None: every pixel), tdic_solve_pois_masked."""
    xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
    p0 = np.ascontiguousarray(p0, np.float64).reshape(-1, 6)
    n = xy.shape[0]
    inp = np.zeros(n, dtype=np.dtype([("x", "<f8"), ("y", "<f8"), ("p0", "<f8", 6), ("confidence", "<f8")]))
    inp["x"], inp["y"], inp["p0"] = xy[:, 0], xy[:, 1], p0
    if confidence is not None:
        inp["confidence"] = confidence
    out = np.zeros(n, dtype=np.dtype([("p", "<f8", 6), ("correlation", "<f8"), ("zncc", "<f8"), ("iterations", "<i4"),
                                      ("status", "i1"), ("valid", "i1"), ("converged", "i1"), ("pad", "i1"),
                                      ("q", "<f8", 6)]))
    if masked:
        rptr, rkeep = _roi_arg(roi, pair.width, pair.height)
        if rptr == "mismatch":
            raise ValueError("roi shape differs from the images")
        ctx.check(ctx.lib.tdic_solve_pois_masked(ctx.handle, pair.handle, C.byref(config), rptr, inp.ctypes.data, n,
                                                 out.ctypes.data, L.HOST, None))
    else:
        ctx.check(ctx.lib.tdic_solve_pois(ctx.handle, pair.handle, C.byref(config), inp.ctypes.data, n,
                                          out.ctypes.data, L.HOST, None))
    return {"p": out["p"].copy(), "q": out["q"].copy(), "correlation": out["correlation"].copy(), "zncc": out["zncc"].copy(),
            "iterations": out["iterations"].copy(), "status": out["status"].copy(),
            "valid": out["valid"].astype(bool), "converged": out["converged"].astype(bool)}


def make_seed(x, y, p, correlation) -> L.Seed:
    s = L.Seed()
    s.x, s.y = float(x), float(y)
    for i in range(6):
        s.p[i] = float(p[i])
    s.correlation = float(correlation)
    s.found = 1
    return s


def propagate(ctx: Context, pair: Pair, config: L.Config, seed: L.Seed, roi=None) -> dict:
    """Propagation over the POI grid (tdic_propagate) in the config's visit order, with host
    outputs; returns the grid dict plus ``points_computed``."""
    gw, gh = L.grid_dims(pair.width, pair.height, config.propagation_spacing)
    arrs, g = _alloc_grid(gw * gh, config.shape_order == 2)
    rptr, rkeep = _roi_arg(roi, pair.width, pair.height)
    if rptr == "mismatch":
        raise ValueError("roi shape differs from the images")
    pc = C.c_int32()
    ctx.check(ctx.lib.tdic_propagate(ctx.handle, pair.handle, C.byref(config), C.byref(seed), rptr, C.byref(g), L.HOST,
                                     C.byref(pc), None))
    out = _finish(arrs)
    out["points_computed"] = pc.value
    out["grid_shape"] = (gh, gw)
    return out


class Batch:
    """Several image pairs propagated in one persistent launch (tdic_batch_*): job j is
    ``propagate(ctx, pairs[j], configs[j], seeds[j], rois[j])`` in the dataflow order.
    ``launch`` only enqueues work on the stream (it can be captured in a CUDA graph);
    ``finish`` waits and returns the points computed per job; ``outputs(j)`` copies job j's grid
    to host arrays (``device_outputs(j)`` gives the device pointers)."""

    def __init__(self, ctx: Context, pairs, configs, seeds, rois=None, stream=None):
        n = len(pairs)
        if not (len(configs) == len(seeds) == n) or (rois is not None and len(rois) != n):
            raise ValueError("pairs, configs, seeds (and rois) must have the same length")
        self.ctx, self.n, self.pairs = ctx, n, list(pairs)
        self._cfgs = (L.Config * n)(*configs)
        self._seeds = (L.Seed * n)(*seeds)
        self._pairs = (C.c_void_p * n)(*[p.handle.value for p in pairs])
        self._rois_keep, roi_ptrs = [], (C.c_void_p * n)()
        for j in range(n):
            r = None if rois is None else rois[j]
            ptr, keep = _roi_arg(r, pairs[j].width, pairs[j].height)
            if ptr == "mismatch":
                raise ValueError("roi shape differs from the images")
            roi_ptrs[j] = ptr
            self._rois_keep.append(keep)
        self._roi_ptrs = roi_ptrs
        self.grid_shapes = []
        for j in range(n):
            gw, gh = L.grid_dims(pairs[j].width, pairs[j].height, configs[j].propagation_spacing)
            self.grid_shapes.append((gh, gw))
        h = C.c_void_p()
        ctx.check(ctx.lib.tdic_batch_create(ctx.handle, n, self._pairs, self._cfgs, self._seeds,
                                            roi_ptrs if rois is not None else None, _stream_ptr(stream), C.byref(h)))
        self.handle = h

    def tune(self, stream=None) -> tuple:
        self.ctx.check(self.ctx.lib.tdic_batch_tune(self.handle, _stream_ptr(stream)))
        return self.config()

    def set_sms(self, sms: int) -> None:
        """Launch on ``sms`` SMs' worth of blocks (0: the whole device), leaving the rest to
        other streams."""
        self.ctx.check(self.ctx.lib.tdic_batch_set_sms(self.handle, int(sms)))

    def config(self) -> tuple:
        """(warps per POI, solver groups per block, staging name) of the launch in use."""
        g, k, st = C.c_int32(), C.c_int32(), C.c_int32()
        self.ctx.check(self.ctx.lib.tdic_batch_config(self.handle, C.byref(g), C.byref(k), C.byref(st)))
        return g.value, k.value, STAGING_NAMES.get(st.value, str(st.value))

    def launch(self, stream=None) -> None:
        self.ctx.check(self.ctx.lib.tdic_batch_launch(self.handle, _stream_ptr(stream)))

    def finish(self, stream=None) -> np.ndarray:
        pc = np.zeros(self.n, np.int32)
        self.ctx.check(self.ctx.lib.tdic_batch_finish(self.handle, _stream_ptr(stream), pc.ctypes.data))
        return pc

    def device_outputs(self, j: int) -> L.GridOut:
        g = L.GridOut()
        self.ctx.check(self.ctx.lib.tdic_batch_outputs(self.handle, int(j), C.byref(g)))
        return g

    def outputs(self, j: int, stream=None) -> dict:
        """Job j's grid as host arrays (the keys of ``propagate``'s result)."""
        gh, gw = self.grid_shapes[j]
        arrs, host = _alloc_grid(gw * gh)
        self.ctx.check(self.ctx.lib.tdic_batch_results(self.handle, int(j), C.byref(host), _stream_ptr(stream)))
        out = _finish(arrs)
        out["grid_shape"] = (gh, gw)
        return out

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.tdic_batch_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prepare(ctx: Context, reference: np.ndarray, deformed: np.ndarray, config: L.Config, roi=None, stream=None):
    """SubsetDIC::compute up to the propagation (tdic_subset_prepare): the pair on the device and
    its seed.  Returns (Pair, Seed); seed.found == 0 is the reference's empty result.  With
    ``truncate_roi_subsets`` the pair holds the images padded by ``padding(config)`` on every side
    and the seed is in padded coordinates: propagate it with ``padded_roi`` and keep the grid
    points inside the image with ``crop_padded`` (what ``compute_config`` returns)."""
    ref = _check_image(reference, "reference")
    de = _check_image(deformed, "deformed")
    if ref.shape != de.shape or ref.dtype != de.dtype:
        raise ValueError("reference and deformed must have the same shape and dtype")
    h, w = ref.shape
    rptr, rkeep = _roi_arg(roi, w, h)
    if rptr == "mismatch":
        raise ValueError("roi shape differs from the images")
    hnd, seed = C.c_void_p(), L.Seed()
    ctx.check(ctx.lib.tdic_subset_prepare(ctx.handle, ref.ctypes.data, de.ctypes.data, w, h, L.DTYPES[ref.dtype.name],
                                          rptr, C.byref(config), _stream_ptr(stream), C.byref(hnd), C.byref(seed)))
    degree = config.degree if config.degree in (1, 3) else 5
    pad = padding(config) if config.truncate_roi_subsets else 0
    return Pair._adopt(ctx, hnd, w + 2 * pad, h + 2 * pad, degree, config.precision, config.border), seed


def padding(config: L.Config) -> int:
    """Pixels added on every side of the images for masked subsets (recommended_subset_padding,
    padding.cpp:11-24; tdic_subset_padding)."""
    return int(L.load().tdic_subset_padding(C.byref(config)))


def padded_roi(roi, w: int, h: int, pad: int) -> np.ndarray:
    """The ROI of the padded pair: 0 in the padding, the caller's mask (all ones if None) inside
    (subset_dic.cpp:58-65)."""
    out = np.zeros((h + 2 * pad, w + 2 * pad), np.uint8)
    out[pad: pad + h, pad: pad + w] = 1 if roi is None else (np.asarray(roi) != 0)
    return out


def crop_padded(result: dict, w: int, h: int, pad: int) -> dict:
    """The grid points of a padded pair's result that lie inside the w x h image, shifted back by
    the padding, in grid order (subset_dic.cpp:84-104), as ``compute_config`` returns them."""
    x = result["x"] - pad
    y = result["y"] - pad
    keep = (x >= 0.0) & (y >= 0.0) & (x < w) & (y < h)
    out = {k: v[keep] for k, v in result.items()}
    out["x"] = x[keep]
    out["y"] = y[keep]
    return out


def integer_search(ctx: Context, pair: Pair, config: L.Config, x, y, roi=None, stream=None) -> dict:
    """IntegerSearchInitializer::estimate at integer points (tdic_integer_search): per point the
    integer displacement u, v, its ZNCC and ok (False where the reference gives no estimate)."""
    xs = np.ascontiguousarray(x, np.int32)
    ys = np.ascontiguousarray(y, np.int32)
    if xs.shape != ys.shape or xs.ndim != 1:
        raise ValueError("x and y must be 1-D arrays of the same length")
    n = len(xs)
    rptr, rkeep = _roi_arg(roi, pair.width, pair.height)
    if rptr == "mismatch":
        raise ValueError("roi shape differs from the images")
    out = {k: np.zeros(n, np.float64) for k in ("u", "v", "zncc")}
    ok = np.zeros(n, np.uint8)
    ctx.check(ctx.lib.tdic_integer_search(ctx.handle, pair.handle, C.byref(config), xs.ctypes.data, ys.ctypes.data,
                                          n, rptr, out["u"].ctypes.data, out["v"].ctypes.data,
                                          out["zncc"].ctypes.data, ok.ctypes.data, _stream_ptr(stream)))
    out["ok"] = ok.astype(bool)
    return out


def select_seed(ctx: Context, lazy_pair: Pair, reference: np.ndarray, config: L.Config, roi=None,
                stream=None) -> L.Seed:
    ref = np.ascontiguousarray(reference, np.float32)
    rptr, rkeep = _roi_arg(roi, lazy_pair.width, lazy_pair.height)
    seed = L.Seed()
    ctx.check(ctx.lib.tdic_select_seed(ctx.handle, lazy_pair.handle, ref.ctypes.data, rptr, C.byref(config),
                                       C.byref(seed), _stream_ptr(stream)))
    return seed
