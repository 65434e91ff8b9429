"""Parity against outputs of the reference itself: the stereo plate case's subset fields.

tests/golden/stereo_plate_fields.npz (made by tests/golden/make_stereo_plate.py from the
reference checkout) holds two subset-DIC fields the reference's own solver wrote
(tests/data/f0b/stereo_plate/fields/left_temporal.npz and reference_disparity.npz of the
reference: L0 -> L4 of camera 1, and L0 -> R0 across the stereo pair, displacements of about
0.3 px and 165 px), the crop of the camera images and ROI they need, and the seed each field is
propagated from.  Configuration: the reference's config/subset_2d.yaml subset section (radius 41,
quintic B-spline, first-order ZNSSD ICGN, 50 iterations, threshold 1e-6, propagation stride 4,
max_znssd 2.0).

The oracle (CPU, FP64) runs left_temporal in the reference's own heap order from the reference's
own seed point, and reference_disparity in the dataflow order on several threads; the GPU path
runs both fields in its default dataflow order, FP64 and FP32-mixed.  Every run must flag exactly
the reference's valid points, and match u, v and the correlation (ZNSSD) on them:

  * FP64 (oracle and GPU): 1e-6 px in u and v and 1e-6 in ZNSSD.  The reference converges every
    point strictly at 1e-6, so results started from other guesses (another visit order, the
    seed's unknown displacement gradients) agree to about the threshold; measured: 3e-7 px.
  * FP32-mixed (GPU): 1e-3 px in u and v, 1e-5 in ZNSSD (the tolerances of the FP32 path).
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stereo_plate_fields.npz")
FIELDS = ("left_temporal", "reference_disparity")
FP64_UV_TOL = 1e-6     # px
FP64_CORR_TOL = 1e-6   # ZNSSD
FP32_UV_TOL = 1e-3     # px
FP32_CORR_TOL = 1e-5   # ZNSSD


@pytest.fixture(scope="module")
def plate():
    d = np.load(GOLDEN)
    return {k: d[k] for k in d.files}


def _images(g, field):
    """read_gray (stereo_3d.py:34-40): float32 pixels divided by the full image's maximum."""
    ref = g["reference"].astype(np.float32) / g["reference_max"]
    de = g[f"{field}_deformed"].astype(np.float32) / g[f"{field}_deformed_max"]
    return np.ascontiguousarray(ref), np.ascontiguousarray(de), np.ascontiguousarray(g["roi"])


def _config(g):
    return json.loads(str(g["config"]))


def compare(g, field, res, uv_tol, corr_tol):
    """The reference's valid set exactly; u, v, correlation on it.  Returns the measured maxima."""
    idx = g[f"{field}_index"]
    valid = np.asarray(res["valid"], bool)
    want = np.zeros(valid.size, bool)
    want[idx] = True
    assert np.array_equal(valid, want), f"{field}: {np.sum(valid != want)} valid flags differ"
    got = {}
    for k in ("u", "v", "correlation"):
        d = np.abs(np.asarray(res[k])[idx] - g[f"{field}_{k}"])
        got[k] = (float(d.max()), float(np.quantile(d, 0.99)))
    print(f"{field}: {idx.size} valid points; max / p99 |du| {got['u'][0]:.2e} / {got['u'][1]:.2e} px, "
          f"|dv| {got['v'][0]:.2e} / {got['v'][1]:.2e} px, |dZNSSD| {got['correlation'][0]:.2e}")
    assert got["u"][0] <= uv_tol and got["v"][0] <= uv_tol
    assert got["correlation"][0] <= corr_tol
    return got


def _oracle_config(oracle, g, mode):
    c = _config(g)
    return oracle.default_config(subset_radius=c["subset"]["radius"],
                                 max_iterations=c["optimization"]["max_iterations"],
                                 convergence_threshold=c["optimization"]["convergence_threshold"],
                                 degree=c["interpolation"]["degree"], criterion=1, shape_order=1, optimizer=0,
                                 propagation_spacing=c["reliability_propagation"]["spacing"],
                                 propagation_max_znssd=c["reliability_propagation"]["max_znssd"],
                                 propagation_mode=mode)


def test_fixture_geometry(plate):
    """The crop's grid is the reference grid's (stride 4 from a multiple of 4) and holds every
    valid point; the seeds lie in the ROI."""
    x0, y0 = plate["origin"]
    assert x0 % 4 == 0 and y0 % 4 == 0
    h, w = plate["reference"].shape
    gw, gh = -(-w // 4), -(-h // 4)
    for f in FIELDS:
        idx = plate[f"{f}_index"]
        assert idx.size == 7654 and idx.max() < gw * gh
        sx, sy = plate[f"{f}_seed"][:2]
        assert plate["roi"][int(round(sy)), int(round(sx))]


@pytest.mark.parametrize("field,mode,threads", [("left_temporal", 1, 1), ("reference_disparity", 2, 8)])
def test_oracle_matches_reference_fields(oracle, plate, field, mode, threads):
    ref, de, roi = _images(plate, field)
    cfg = _oracle_config(oracle, plate, mode)
    coef = oracle.prefilter(de, cfg.degree, cfg.border, True)
    sx, sy, u, v, corr = plate[f"{field}_seed"]
    seed = oracle.make_seed(sx, sy, [u, v, 0.0, 0.0, 0.0, 0.0], corr)
    res = oracle.propagate(ref, coef, cfg, seed, roi=roi, threads=threads)
    compare(plate, field, res, FP64_UV_TOL, FP64_CORR_TOL)


@pytest.mark.gpu
@pytest.mark.parametrize("field", FIELDS)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_matches_reference_fields(plate, field, precision):
    from traditional_dic_gb300 import subset as S, _lib as L
    ref, de, roi = _images(plate, field)
    cfg = S.config_from_dict(dict(_config(plate), gpu={"precision": precision}))
    ctx = S.default_context()
    pair = S.Pair(ctx, ref, de, degree=cfg.degree, precision=cfg.precision)
    sx, sy, u, v, corr = plate[f"{field}_seed"]
    seed = S.make_seed(sx, sy, [u, v, 0.0, 0.0, 0.0, 0.0], corr)
    res = S.propagate(ctx, pair, cfg, seed, roi=roi)
    pair.close()
    if precision == "fp64":
        compare(plate, field, res, FP64_UV_TOL, FP64_CORR_TOL)
    else:
        compare(plate, field, res, FP32_UV_TOL, FP32_CORR_TOL)
