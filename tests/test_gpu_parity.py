"""GPU parity: the CUDA path through the C ABI against the FP64 CPU oracle.

Tolerances (stated by the task for floating point): displacement 1e-3 px, ZNCC 1e-5,
gradient parameters 1e-5, convergence flags identical on >= 99.9% of POIs.  The FP64 build
is held to much tighter bounds (same arithmetic up to summation order).
"""
import numpy as np
import pytest

from conftest import small_speckle

pytestmark = pytest.mark.gpu

U_TOL = 1e-3      # px
G_TOL = 1e-5      # displacement gradients
Z_TOL = 1e-5      # ZNCC
FLAG_AGREE = 0.999


def _cfg(S, **kw):
    c = S.config_from_dict({"interpolation": {"degree": kw.pop("degree", 3)}})
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("degree", [1, 3, 5])
@pytest.mark.parametrize("precision", [0, 1])
def test_prefilter_matches_oracle(oracle, gpu_ctx, degree, precision):
    from traditional_dic_gb300 import subset as S
    p = small_speckle((70, 90), n=200)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=degree, border=3, precision=precision)
    got = pair.coefficients().astype(np.float64)
    want = oracle.prefilter(p.deformed.astype(np.float32), degree, 3, True)
    tol = 1e-11 if precision == 1 else 2e-5
    assert np.max(np.abs(got - want)) <= tol * max(1.0, np.abs(want).max())


def test_lazy_coefficients_match_oracle(oracle, gpu_ctx):
    from traditional_dic_gb300 import subset as S
    p = small_speckle((40, 50), n=60)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=5, border=4, exact=False, precision=1)
    want = oracle.prefilter(p.deformed.astype(np.float32), 5, 4, False)
    assert np.array_equal(pair.coefficients(), want)


def test_reference_gradient_matches_oracle(oracle, gpu_ctx):
    from traditional_dic_gb300 import subset as S
    p = small_speckle((33, 47), n=50)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed)
    gx, gy = pair.reference_gradient()
    ox, oy = oracle.reference_gradient(p.reference.astype(np.float32))
    assert np.array_equal(gx, ox) and np.array_equal(gy, oy)


def _poi_case(p, step=6, r=8, jitter=0.3, seed=3):
    rng = np.random.default_rng(seed)
    h, w = p.reference.shape
    ys, xs = np.mgrid[r:h - r:step, r:w - r:step]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.float64)
    u, v, ux, uy, vx, vy = p.truth(xy[:, 0], xy[:, 1])
    p0 = np.stack([np.round(u) + rng.uniform(-jitter, jitter, u.size), np.round(v) + rng.uniform(-jitter, jitter, u.size),
                   0 * u, 0 * u, 0 * u, 0 * u], 1)
    return xy, p0


@pytest.mark.parametrize("optimizer", [0, 1])
@pytest.mark.parametrize("degree", [3, 5])
def test_solve_pois_fp64_matches_oracle(oracle, gpu_ctx, optimizer, degree):
    from traditional_dic_gb300 import subset as S
    p = small_speckle((96, 96), n=240)
    cfg = _cfg(S, degree=degree, subset_radius=8, max_iterations=25, convergence_threshold=1e-6, optimizer=optimizer,
               precision=1)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=degree, precision=1)
    xy, p0 = _poi_case(p)
    got = S.solve_pois(gpu_ctx, pair, cfg, xy, p0)
    coef = oracle.prefilter(p.deformed.astype(np.float32), degree, 3, True)
    want = oracle.solve_pois(p.reference, coef, oracle.as_config(cfg), xy, p0,
                             gradients=oracle.reference_gradient(p.reference.astype(np.float32)))
    assert np.array_equal(got["status"], want["status"])
    same_it = got["iterations"] == want["iterations"]
    assert same_it.mean() >= 0.99
    ok = same_it & (want["status"] == 0)
    assert np.max(np.abs(got["p"][ok] - want["p"][ok])) < 1e-8
    assert np.max(np.abs(got["correlation"][ok] - want["correlation"][ok])) < 1e-10


@pytest.mark.parametrize("optimizer", [0, 1])
def test_solve_pois_fp32_within_tolerance(oracle, gpu_ctx, optimizer):
    from traditional_dic_gb300 import subset as S
    p = small_speckle((96, 96), n=240)
    cfg = _cfg(S, degree=3, subset_radius=8, max_iterations=20, convergence_threshold=1e-3, optimizer=optimizer,
               precision=0)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, precision=0)
    xy, p0 = _poi_case(p)
    got = S.solve_pois(gpu_ctx, pair, cfg, xy, p0)
    coef = oracle.prefilter(p.deformed.astype(np.float32), 3, 3, True)
    want = oracle.solve_pois(p.reference, coef, oracle.as_config(cfg), xy, p0)
    assert np.mean(got["valid"] == want["valid"]) >= FLAG_AGREE
    ok = got["valid"] & want["valid"]
    assert np.max(np.abs(got["p"][ok, :2] - want["p"][ok, :2])) <= U_TOL
    zg = np.clip(1 - 0.5 * got["correlation"][ok], -1, 1)
    zw = np.clip(1 - 0.5 * want["correlation"][ok], -1, 1)
    assert np.max(np.abs(zg - zw)) <= Z_TOL


def test_solve_pois_edge_statuses(oracle, gpu_ctx):
    """Subset outside the image, warp leaving the image, flat subset, zero iterations."""
    from traditional_dic_gb300 import subset as S
    p = small_speckle((64, 64), n=100)
    ref = p.reference.copy()
    ref[:20, :20] = 77  # flat patch -> NumericalFailure
    pair = S.Pair(gpu_ctx, ref, p.deformed, degree=3, precision=1)
    xy = np.array([[3.0, 30.0], [30.0, 30.0], [10.0, 10.0], [32.0, 32.0], [31.5, 32.5]])
    p0 = np.zeros((5, 6))
    p0[1, 0] = 40.0  # warped out of the image -> InvalidInput
    cfg = _cfg(S, degree=3, subset_radius=8, max_iterations=10, precision=1)
    got = S.solve_pois(gpu_ctx, pair, cfg, xy, p0, confidence=np.full(5, 0.25))
    coef = oracle.prefilter(p.deformed.astype(np.float32), 3, 3, True)
    want = oracle.solve_pois(ref, coef, oracle.as_config(cfg), xy, p0, confidence0=np.full(5, 0.25))
    assert list(got["status"]) == list(want["status"])
    assert got["status"][0] == 2 and got["status"][1] == 2 and got["status"][2] == 3
    assert np.allclose(got["correlation"][:3], 0.25)
    cfg0 = _cfg(S, degree=3, subset_radius=8, max_iterations=0, precision=1)
    z = S.solve_pois(gpu_ctx, pair, cfg0, xy[3:4], p0[3:4])
    assert z["status"][0] == 1 and not z["valid"][0] and z["iterations"][0] == 0


def _seed_from_oracle(oracle, p, cfg):
    seed, _ = oracle.select_seed(p.reference, p.deformed, oracle.as_config(cfg))
    assert seed.found
    return seed


@pytest.mark.parametrize("mode", [0, 2])
@pytest.mark.parametrize("precision", [1, 0])
def test_propagate_matches_oracle_same_order(oracle, gpu_ctx, workload0, precision, mode):
    """GPU propagation against the oracle run in the same visit order (0 frontier waves,
    2 dataflow + wave clean-up)."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    cfg.precision = precision
    cfg.propagation_mode = mode
    oseed = _seed_from_oracle(oracle, p, cfg)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, precision=precision)
    seed = S.make_seed(oseed.x, oseed.y, list(oseed.p), oseed.correlation)
    got = S.propagate(gpu_ctx, pair, cfg, seed)
    ocfg = oracle.as_config(cfg)
    ocfg.propagation_mode = mode
    coef = oracle.prefilter(p.deformed.astype(np.float32), 3, 3, True)
    want = oracle.propagate(p.reference, coef, ocfg, oseed)
    assert got["points_computed"] == want["points_computed"] or precision == 0
    assert np.array_equal(got["x"], want["x"]) and np.array_equal(got["y"], want["y"])
    assert np.mean(got["valid"] == want["valid"]) >= FLAG_AGREE
    both = got["valid"] & want["valid"]
    tol = 1e-7 if precision == 1 else U_TOL
    assert np.max(np.abs(got["u"][both] - want["u"][both])) <= tol
    assert np.max(np.abs(got["v"][both] - want["v"][both])) <= tol


def test_compute_matches_oracle_pipeline(oracle, gpu_ctx, workload0):
    """Whole drop-in path (seed selection + propagation) against the oracle's reference pipeline
    (serial reliability-guided heap order)."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    got, seed = S.compute(p.reference, p.deformed, G.WORKLOAD0_CONFIG, return_seed=True)
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    want = oracle.subset_compute(p.reference, p.deformed, oracle.as_config(cfg) if False else _heap(oracle, cfg))
    assert seed.found and want["seed"].found
    assert (seed.x, seed.y) == (want["seed"].x, want["seed"].y)
    assert abs(seed.p[0] - want["seed"].p[0]) <= U_TOL and abs(seed.p[1] - want["seed"].p[1]) <= U_TOL
    assert len(got["x"]) == len(want["x"])
    assert np.mean(got["valid"] == want["valid"]) >= FLAG_AGREE
    both = got["valid"] & want["valid"]
    d = np.hypot(got["u"][both] - want["u"][both], got["v"][both] - want["v"][both])
    # visit order differs (frontier waves vs serial heap): report, bound loosely
    assert np.quantile(d, 0.9) <= U_TOL
    assert d.max() <= 10 * U_TOL


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_compute_heap_order_matches_oracle_pipeline(oracle, gpu_ctx, workload0, precision):
    """The drop-in path in the reference's own visit order (propagation "heap": seed selection,
    then the heap loop reproduced on the device) against the oracle's reference pipeline: the
    same seed, the same grid, and results within FP32 rounding (FP64: to 1e-7 px, flags and
    iteration counts identical)."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    conf = dict(G.WORKLOAD0_CONFIG, gpu={"precision": precision, "propagation": "heap"})
    got, seed = S.compute(p.reference, p.deformed, conf, return_seed=True)
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    want = oracle.subset_compute(p.reference, p.deformed, _heap(oracle, cfg))
    assert seed.found and want["seed"].found
    assert (seed.x, seed.y) == (want["seed"].x, want["seed"].y)
    assert len(got["x"]) == len(want["x"])
    both = got["valid"] & want["valid"]
    d = np.hypot(got["u"][both] - want["u"][both], got["v"][both] - want["v"][both])
    if precision == "fp64":
        assert np.array_equal(got["valid"], want["valid"])
        assert d.max() <= 1e-7
        return
    assert np.mean(got["valid"] == want["valid"]) >= FLAG_AGREE
    assert np.mean(d <= U_TOL) >= 0.999 and np.quantile(d, 0.99) <= 1e-5


@pytest.mark.parametrize("with_roi", [False, True])
def test_select_seed_matches_oracle(oracle, gpu_ctx, workload0, with_roi):
    """Seed selection (sampled candidate points, k-means, integer search, subpixel refinement)
    against the oracle; 256^2 has more candidate points than the k-means sample limit."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    roi = None
    if with_roi:
        yy, xx = np.mgrid[:256, :256]
        roi = (((xx - 150) ** 2 + (yy - 120) ** 2) < 90 ** 2) | ((xx < 60) & (yy > 100))
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    lazy = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, exact=False)
    got = S.select_seed(gpu_ctx, lazy, p.reference.astype(np.float32), cfg, roi=roi)
    want, _ = oracle.select_seed(p.reference, p.deformed, oracle.as_config(cfg), roi=roi)
    assert got.found and want.found
    assert (got.x, got.y) == (want.x, want.y)
    assert abs(got.p[0] - want.p[0]) <= U_TOL and abs(got.p[1] - want.p[1]) <= U_TOL
    if roi is not None:
        assert roi[int(got.y), int(got.x)]


def _search_points(oracle, p, cfg, roi):
    """The oracle's seed candidates plus points at and near the image border (no estimate, or a
    search window cut by the border)."""
    _, cand = oracle.select_seed(p.reference, p.deformed, oracle.as_config(cfg), roi=roi)
    h, w = p.reference.shape
    r = cfg.is_subset_radius
    extra = [(r, r), (r - 1, 40), (w - 1 - r, h // 2), (w - r, h // 3), (w // 2, h - 1 - r), (0, 0),
             (r + 3, h - r - 4), (w // 3, r + 1)]
    xs = np.array([int(round(c[0])) for c in cand] + [e[0] for e in extra], np.int32)
    ys = np.array([int(round(c[1])) for c in cand] + [e[1] for e in extra], np.int32)
    return xs, ys, len(cand)


@pytest.mark.parametrize("with_roi", [False, True])
def test_integer_search_matches_oracle(oracle, gpu_ctx, workload0, with_roi):
    """IntegerSearchInitializer::estimate point by point (tdic_integer_search): the integer
    displacement exactly, its FP64 ZNCC to 1e-12 and the no-estimate points, at the oracle's seed
    candidates and at the border; with a ROI, the masked search."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    roi = None
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    if with_roi:
        yy, xx = np.mgrid[:256, :256]
        roi = (((xx - 150) ** 2 + (yy - 120) ** 2) < 90 ** 2) | ((xx < 60) & (yy > 100))
        cfg.truncate_roi_subsets = 1
    xs, ys, ncand = _search_points(oracle, p, cfg, roi)
    assert ncand > 8
    for exact in (False, True):   # either prefilter: the search reads the pair's float32 images
        pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, exact=exact)
        got = S.integer_search(gpu_ctx, pair, cfg, xs, ys, roi=roi)
        pair.close()
        for i in range(len(xs)):
            want = oracle.integer_search(p.reference, p.deformed, oracle.as_config(cfg), xs[i], ys[i], roi=roi)
            assert got["ok"][i] == (want is not None), (exact, i, xs[i], ys[i])
            if want is None:
                continue
            assert (got["u"][i], got["v"][i]) == (want[0], want[1]), (exact, i)
            assert abs(got["zncc"][i] - want[2]) <= 1e-12, (exact, i)
        assert got["ok"][:ncand].all()


def test_integer_search_refuses_more_points_than_a_grid_row(gpu_ctx, workload0):
    """One coarse-grid row per point: more than 65535 points in one call is refused up front."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S, _lib as L
    p = workload0
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, exact=False)
    pts = np.full(65536, 128, np.int32)
    with pytest.raises(L.TdicError, match="at most 65535 points"):
        S.integer_search(gpu_ctx, pair, cfg, pts, pts)
    got = S.integer_search(gpu_ctx, pair, cfg, pts[:3], pts[:3])   # the context stays usable
    assert len(set(got["ok"])) == 1 and len(set(got["u"])) == 1 and len(set(got["v"])) == 1
    pair.close()


def _heap(oracle, cfg):
    c = oracle.as_config(cfg)
    c.propagation_mode = 1
    return c


def test_compute_empty_results(gpu_ctx):
    from traditional_dic_gb300 import subset as S
    p = small_speckle((64, 64), n=80)
    r = S.compute(p.reference, p.deformed[:, :60].copy(), None)
    assert all(len(r[k]) == 0 for k in S.RESULT_KEYS)
    r = S.compute(p.reference, p.deformed, {"initialization": {"integer_search": {"sift_enabled": True}}})
    assert len(r["x"]) == 0


@pytest.mark.parametrize("precision", [0, 1])
def test_solve_pois_large_radius(oracle, gpu_ctx, precision):
    """r = 25 (1961 samples): shared-memory staging sized per radius, adaptive groups per CTA."""
    from traditional_dic_gb300 import subset as S
    p = small_speckle((128, 128), n=420)
    cfg = _cfg(S, degree=5, subset_radius=25, max_iterations=20, convergence_threshold=1e-3, precision=precision)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=5, precision=precision)
    xy, p0 = _poi_case(p, step=13, r=25)
    got = S.solve_pois(gpu_ctx, pair, cfg, xy, p0)
    coef = oracle.prefilter(p.deformed.astype(np.float32), 5, 3, True)
    want = oracle.solve_pois(p.reference, coef, oracle.as_config(cfg), xy, p0)
    assert np.mean(got["valid"] == want["valid"]) >= FLAG_AGREE
    ok = got["valid"] & want["valid"]
    tol = 1e-8 if precision == 1 else U_TOL
    assert np.max(np.abs(got["p"][ok, :2] - want["p"][ok, :2])) <= tol
