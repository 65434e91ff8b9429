"""CPU checks of the C ABI boundary: the library builds and loads, exports every function that
include/tdic_gb300.h declares, and the host-side config mirror behaves like the reference's
pybind parser (bind_subset.cpp:158-248).  No device call is made here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "tdic_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tdic_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(pkg):
    from traditional_dic_gb300 import _lib as L
    lib = L.load()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(L.SIGNATURES)


def test_struct_layouts_match_header(pkg, oracle):
    from traditional_dic_gb300 import _lib as L
    assert C.sizeof(L.Config) == 160
    assert C.sizeof(L.Config) == C.sizeof(oracle.Config)
    assert [f for f, _ in L.Config._fields_] == [f for f, _ in oracle.Config._fields_]
    assert C.sizeof(L.PoiIn) == 72 and C.sizeof(L.PoiOut) == 120 and C.sizeof(L.Seed) == 80
    assert C.sizeof(L.GridOut) == 20 * C.sizeof(C.c_void_p)
    assert C.sizeof(oracle.PoiResult) == 112 and C.sizeof(oracle.GridOut) == 19 * C.sizeof(C.c_void_p)


def test_defaults_match_reference_cpp_defaults(pkg, oracle):
    from traditional_dic_gb300 import _lib as L
    ours = L.default_config().as_dict()
    ref = {k: getattr(oracle.default_config(), k) for k, _ in oracle.CONFIG_FIELDS}
    for k in ours:
        if k in ("propagation_mode", "precision", "staging"):
            continue
        assert ours[k] == ref[k], k
    # subset_config.hpp:33-50, seed_config.hpp:32-68, bspline.hpp:62-63
    assert (ours["subset_radius"], ours["max_iterations"], ours["degree"], ours["propagation_spacing"]) == (15, 30, 5, 5)
    assert ours["seed_count"] == 256 and ours["seed_max_znssd"] == 0.2 and ours["is_search_radius"] == 30


def test_config_from_dict_mirrors_pybind(pkg):
    from traditional_dic_gb300 import subset as S
    c = S.config_from_dict({"interpolation": {"degree": 3}, "optimization": {"method": "fgn", "max_iterations": 7},
                            "reliability_propagation": {"spacing": 4, "max_znssd": 0.25}})
    assert (c.degree, c.optimizer, c.max_iterations, c.propagation_spacing, c.propagation_max_znssd) == (3, 1, 7, 4, 0.25)
    assert S.config_from_dict({"interpolation": {"degree": 2}}).degree == 5     # only 1 and 3 are mapped
    assert S.config_from_dict({"interpolation": {"degree": 1}}).degree == 1
    assert S.config_from_dict({"correlation": {"criterion": "ssd"}}).criterion == 0
    assert S.config_from_dict({"shape_function": {"order": "2"}}).shape_order == 2
    assert S.config_from_dict({"gpu": {"precision": "fp64"}}).precision == 1
    for bad in ({"optimization": {"method": "lm"}}, {"correlation": {"criterion": "ncc"}},
                {"initialization": {"method": "sift"}}, {"shape_function": {"order": "3"}},
                {"subset": {"radius": 2.5}}, {"gpu": {"precision": "fp16"}}):
        with pytest.raises(RuntimeError):
            S.config_from_dict(bad)
    assert S.config_from_dict({"optimization": {"convergence_threshold": 1}}).convergence_threshold == 1.0


def test_argument_errors_before_any_device_call(pkg):
    from traditional_dic_gb300 import subset as S
    with pytest.raises(RuntimeError, match="2D numpy array"):
        S.compute(np.zeros((4, 4, 3), np.float32), np.zeros((4, 4, 3), np.float32))
    with pytest.raises(RuntimeError, match="float32 or float64"):
        S.compute([[1.0]], np.zeros((4, 4), np.float32))
    with pytest.raises(RuntimeError, match="config must be a dict"):
        S.compute(np.zeros((4, 4), np.float32), np.zeros((4, 4), np.float32), config="x.yaml")
    with pytest.raises(ValueError):
        S.subset(np.zeros((4, 4), np.float32), np.zeros((4, 5), np.float32))


def test_grid_dims(pkg):
    from traditional_dic_gb300 import _lib as L
    assert L.grid_dims(2048, 2048, 4) == (410, 410)
    assert L.grid_dims(5120, 5120, 2) == (1707, 1707)
    assert L.grid_dims(7, 3, -4) == (7, 3)
    assert L.grid_dims(5, 5, 2 ** 31 - 1) == (1, 1) and L.grid_dims(2 ** 31 - 1, 1, 2 ** 31 - 2) == (1, 1)


def test_truncation_geometry_matches_oracle(pkg, oracle):
    """recommended_subset_padding (padding.cpp:28-36) and the cropped output grid of
    SubsetDIC::compute with truncate_roi_subsets (subset_dic.cpp:53-104): the library's host
    functions against the oracle over a sweep of image sizes, spacings and radii."""
    from traditional_dic_gb300 import _lib as L
    rng = np.random.default_rng(11)
    for _ in range(300):
        cfg = L.default_config()
        cfg.truncate_roi_subsets = int(rng.integers(0, 2))
        cfg.subset_radius = int(rng.integers(1, 40))
        cfg.is_subset_radius = int(rng.integers(-2, 40))
        cfg.sp_subset_radius = int(rng.integers(-2, 40))
        cfg.is_search_radius = int(rng.integers(-5, 80))
        cfg.border = int(rng.integers(-2, 8))
        cfg.propagation_spacing = int(rng.integers(-3, 12))
        w, h = int(rng.integers(0, 300)), int(rng.integers(0, 300))
        pad = L.load().tdic_subset_padding(C.byref(cfg))
        # the library reports the padding subset_compute applies: none without truncation
        assert pad == (oracle.subset_padding(cfg) if cfg.truncate_roi_subsets else 0)
        got = L.subset_grid_dims(w, h, cfg)
        assert got == oracle.truncated_grid_dims(w, h, cfg)
        step = max(0, cfg.propagation_spacing) + 1
        # the points kept are exactly the padded grid's points x = g * step - pad inside [0, w)
        for n, g in ((w, got[0]), (h, got[1])):
            gp = -(-(n + 2 * pad) // step)
            assert g == sum(1 for k in range(gp) if 0 <= k * step - pad < n)
        if not cfg.truncate_roi_subsets:
            assert got == L.grid_dims(w, h, cfg.propagation_spacing)


def test_context_creation_failure_reports_its_cause(pkg):
    """Without a usable device tdic_ctx_create fails, and tdic_last_error(NULL) carries the CUDA
    message of that failure (there is no context to hold it); the facade puts it in its error."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is visible: context creation succeeds")
    from traditional_dic_gb300 import _lib as L, subset as S
    lib = L.load()
    h = C.c_void_p()
    assert lib.tdic_ctx_create(0, C.byref(h)) == L.TDIC_CUDA_ERROR and not h.value
    msg = lib.tdic_last_error(None).decode()
    assert msg != "null context" and "cudaSetDevice" in msg
    with pytest.raises(L.TdicError, match="cudaSetDevice"):
        S.Context(0)


def test_pair_update_checks_both_images(pkg):
    """Pair.update hands both buffers to the library under one dtype: images of another shape,
    dtype or memory kind are refused before any library call."""
    from traditional_dic_gb300 import subset as S
    pair = S.Pair._adopt(None, C.c_void_p(), 16, 12, 3, 0, 3)   # no device: the checks run first
    u8 = np.zeros((12, 16), np.uint8)
    with pytest.raises(ValueError, match="same dtype"):
        pair.update(u8, u8.astype(np.float32))
    with pytest.raises(ValueError, match="shape"):
        pair.update(u8, np.zeros((12, 15), np.uint8))
    with pytest.raises(ValueError, match="shape"):
        pair.update(np.zeros((13, 16), np.uint8), np.zeros((13, 16), np.uint8))
