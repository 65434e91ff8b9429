"""Shared-memory staging modes of the first-order ZNSSD solves (tdic_config.staging): full, lean
(reference values and gradients re-read from the staged reference window) and lean without the
coefficient window (spline stencils read from the coefficient image).  The mode is a layout
choice only, so every output of every point must be the same bit for bit, for ICGN and FGN, in
FP32-mixed and FP64, through the propagation and the per-POI solve."""
import numpy as np
import pytest

MODES = ("lean", "lean_no_window")
KEYS = ("u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "zncc", "valid", "status", "iterations",
        "converged")


def _config(G, precision, optimizer, staging):
    from traditional_dic_gb300 import subset as S
    d = dict(G.WORKLOAD0_CONFIG, gpu={"precision": precision, "staging": staging})
    d["optimization"] = dict(d["optimization"], method=optimizer)
    return S.config_from_dict(d)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("optimizer", ["icgn", "fgn"])
def test_staging_modes_give_identical_propagations(gpu_ctx, oracle, workload0, precision, optimizer):
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    cfg = _config(G, precision, optimizer, "full")
    seed_o, _ = oracle.select_seed(p.reference, p.deformed, oracle.as_config(cfg))
    seed = S.make_seed(seed_o.x, seed_o.y, list(seed_o.p), seed_o.correlation)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, precision=cfg.precision)
    want = S.propagate(gpu_ctx, pair, cfg, seed)
    assert want["points_computed"] > 100
    for mode in MODES:
        got = S.propagate(gpu_ctx, pair, _config(G, precision, optimizer, mode), seed)
        assert got["points_computed"] == want["points_computed"], mode
        for k in KEYS:
            assert np.array_equal(got[k], want[k], equal_nan=True), (mode, k)
    pair.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_staging_modes_give_identical_solves(gpu_ctx, workload0, precision):
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, precision=1 if precision == "fp64" else 0)
    ys, xs = np.mgrid[12:244:9, 12:244:9]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.float64)
    p0 = np.zeros((len(xy), 6))
    p0[:, 0] = np.round(2.3 + 0.001 * xy[:, 0])
    p0[:, 1] = np.round(-1.7 - 0.0005 * xy[:, 1])
    for optimizer in ("icgn", "fgn"):
        want = S.solve_pois(gpu_ctx, pair, _config(G, precision, optimizer, "full"), xy, p0)
        assert np.sum(want["valid"]) > 0.9 * len(xy)
        for mode in MODES:
            got = S.solve_pois(gpu_ctx, pair, _config(G, precision, optimizer, mode), xy, p0)
            for k in ("p", "correlation", "iterations", "status", "valid", "converged"):
                assert np.array_equal(got[k], want[k], equal_nan=True), (optimizer, mode, k)
    pair.close()


@pytest.mark.gpu
def test_fp64_large_radius_needs_lean_staging(gpu_ctx, workload0):
    """Radius 41 in FP64 (the reference's own subset_2d.yaml radius): four per-sample arrays of
    5281 doubles and the FP64 coefficient window exceed a block's shared memory, so full staging
    is refused and the automatic choice runs lean."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S, _lib as L
    rng = np.random.default_rng(5)
    img = (rng.random((200, 200)) * 200).astype(np.float32)
    pair = S.Pair(gpu_ctx, img, img, degree=5, precision=L.FP64)
    xy = np.array([[100.0, 100.0]])
    p0 = np.zeros((1, 6))
    d = dict(G.WORKLOAD0_CONFIG, subset={"radius": 41}, interpolation={"degree": 5})
    full = S.config_from_dict(dict(d, gpu={"precision": "fp64", "staging": "full"}))
    with pytest.raises(L.TdicError) as e:
        S.solve_pois(gpu_ctx, pair, full, xy, p0)
    assert e.value.status == L.TDIC_UNSUPPORTED
    auto = S.config_from_dict(dict(d, gpu={"precision": "fp64"}))
    r = S.solve_pois(gpu_ctx, pair, auto, xy, p0)
    assert r["valid"][0] and r["converged"][0] and np.max(np.abs(r["p"][0])) < 1e-9
    pair.close()
