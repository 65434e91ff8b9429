"""Golden vectors (tests/golden/*.npz, made by tests/golden/make_golden.py from an independent
numpy transcription of the reference): the C++ oracle (CPU) and the GPU path (GPU) must reproduce
the B-spline coefficients and the per-POI results of every solver route, full and masked; the
oracle must reproduce whole heap-order propagations over the grid and the seed selection (k-means
candidates, integer search, subpixel refinement), with and without a ROI, and the whole
SubsetDIC::compute with truncated subsets over padded images."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_icgn_256.npz")
P_TOL = 1e-8       # px and displacement gradients between two FP64 transcriptions
U_TOL = 1e-3       # px, FP32-mixed path


@pytest.fixture(scope="module")
def golden():
    d = np.load(GOLDEN)
    return {k: d[k] for k in d.files}


def _inputs(g):
    pois = g["pois"]
    xy = pois[:, :2]
    p0 = np.zeros((len(pois), 6))
    p0[:, :2] = pois[:, 2:4]
    return xy, p0


def _config(g, make_default):
    degree, border, radius, max_iter, thr = g["settings"]
    cfg = make_default()
    cfg.subset_radius, cfg.max_iterations, cfg.convergence_threshold = int(radius), int(max_iter), float(thr)
    cfg.degree, cfg.border, cfg.optimizer = int(degree), int(border), 0
    return cfg


def _check(got_p, got_iters, got_status, got_corr, g, tol):
    res = g["results"]
    want_p, want_corr = res[:, :6], res[:, 6]
    want_iters, want_status = res[:, 7].astype(int), res[:, 8].astype(int)
    assert np.array_equal(np.asarray(got_status, int), want_status)
    ok = want_status == 0
    assert np.array_equal(np.asarray(got_iters, int)[ok], want_iters[ok])
    assert np.max(np.abs(got_p[ok] - want_p[ok])) <= tol
    assert np.max(np.abs(np.asarray(got_corr)[ok] - want_corr[ok])) <= max(tol, 1e-9)


def test_oracle_coefficients_match_golden(oracle, golden):
    degree, border = int(golden["settings"][0]), int(golden["settings"][1])
    coef = oracle.prefilter(golden["deformed"].astype(np.float32), degree, border, True)
    assert np.max(np.abs(coef[:40, :40] - golden["coef_crop"])) <= 1e-10


def test_oracle_icgn_matches_golden(oracle, golden):
    cfg = _config(golden, oracle.default_config)
    coef = oracle.prefilter(golden["deformed"].astype(np.float32), cfg.degree, cfg.border, True)
    xy, p0 = _inputs(golden)
    ref = golden["reference"].astype(np.float32)
    r = oracle.solve_pois(ref, coef, cfg, xy, p0, gradients=oracle.reference_gradient(ref))
    _check(r["p"], r["iterations"], r["status"], r["correlation"], golden, P_TOL)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [1, 0])
def test_gpu_icgn_matches_golden(gpu_ctx, golden, precision):
    from traditional_dic_gb300 import subset as S, _lib as L
    cfg = _config(golden, L.default_config)
    cfg.precision = precision
    pair = S.Pair(gpu_ctx, golden["reference"], golden["deformed"], degree=cfg.degree, border=cfg.border,
                  precision=precision)
    coef = pair.coefficients()
    if precision == 1:
        assert np.max(np.abs(coef[:40, :40] - golden["coef_crop"])) <= 1e-10
    xy, p0 = _inputs(golden)
    r = S.solve_pois(gpu_ctx, pair, cfg, xy, p0)
    if precision == 1:
        _check(r["p"], r["iterations"], r["status"], r["correlation"], golden, P_TOL)
    else:
        res = golden["results"]
        ok = res[:, 8] == 0
        assert np.array_equal(r["status"], res[:, 8].astype(int))
        assert np.max(np.abs(r["p"][ok, :2] - res[ok, :2])) <= U_TOL
    pair.close()


# ---- the other solver routes (tests/golden/subset_variants_256.npz) --------------------------
VARIANTS_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_variants_256.npz")
VARIANTS = [("icgn1_ssd", 0, 1, 0), ("icgn2_znssd", 0, 2, 1), ("icgn2_ssd", 0, 2, 0),
            ("fgn1_ssd", 1, 1, 0), ("fgn2_znssd", 1, 2, 1), ("fgn2_ssd", 1, 2, 0)]
Q_TOL = 1e-9       # second-order terms (px / px^2) between two FP64 transcriptions


@pytest.fixture(scope="module")
def variants():
    d = np.load(VARIANTS_FILE)
    return {k: d[k] for k in d.files}


def _variant_config(g, make_default, opt, order, crit):
    degree, border, radius, max_iter, thr = g["settings"]
    cfg = make_default()
    cfg.subset_radius, cfg.max_iterations, cfg.convergence_threshold = int(radius), int(max_iter), float(thr)
    cfg.degree, cfg.border = int(degree), int(border)
    cfg.optimizer, cfg.shape_order, cfg.criterion = opt, order, crit
    return cfg


def _variant_inputs(g, tag):
    pois = g[f"pois_{tag}"]
    p0 = np.zeros((len(pois), 6))
    p0[:, :2] = pois[:, 2:4]
    return pois[:, :2], p0


def _check_variant(r, want, p_tol, q_tol, corr_rtol):
    want_p, want_q, want_corr = want[:, :6], want[:, 6:12], want[:, 12]
    want_iters, want_status = want[:, 13].astype(int), want[:, 14].astype(int)
    assert np.array_equal(np.asarray(r["status"], int), want_status)
    ok = want_status == 0
    assert np.array_equal(np.asarray(r["iterations"], int)[ok], want_iters[ok])
    assert np.max(np.abs(r["p"][ok] - want_p[ok])) <= p_tol
    assert np.max(np.abs(r["q"][ok] - want_q[ok])) <= q_tol
    c = np.asarray(r["correlation"])[ok]
    assert np.max(np.abs(c - want_corr[ok]) / np.maximum(1.0, np.abs(want_corr[ok]))) <= corr_rtol


@pytest.mark.parametrize("tag", ["a", "b"])
@pytest.mark.parametrize("name,opt,order,crit", VARIANTS)
def test_oracle_variants_match_golden(oracle, variants, name, opt, order, crit, tag):
    cfg = _variant_config(variants, oracle.default_config, opt, order, crit)
    ref = variants[f"reference_{tag}"].astype(np.float32)
    coef = oracle.prefilter(variants[f"deformed_{tag}"].astype(np.float32), cfg.degree, cfg.border, True)
    xy, p0 = _variant_inputs(variants, tag)
    r = oracle.solve_pois(ref, coef, cfg, xy, p0, gradients=oracle.reference_gradient(ref))
    _check_variant(r, variants[f"{name}_{tag}"], P_TOL, Q_TOL, 1e-9)


# ---- masked subsets (tests/golden/subset_masked_256.npz) ------------------------------------
MASKED_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_masked_256.npz")
MASKED = [("icgn1_znssd", 0, 1, 1), ("icgn2_ssd", 0, 2, 0), ("fgn1_ssd", 1, 1, 0), ("fgn2_znssd", 1, 2, 1)]


@pytest.fixture(scope="module")
def masked():
    d = np.load(MASKED_FILE)
    return {k: d[k] for k in d.files}


@pytest.mark.parametrize("name,opt,order,crit", MASKED)
def test_oracle_masked_match_golden(oracle, masked, golden, name, opt, order, crit):
    cfg = _variant_config(masked, oracle.default_config, opt, order, crit)
    cfg.truncate_roi_subsets = 1
    ref = golden["reference"].astype(np.float32)
    coef = oracle.prefilter(golden["deformed"].astype(np.float32), cfg.degree, cfg.border, True)
    pois = masked["pois"]
    p0 = np.zeros((len(pois), 6))
    p0[:, :2] = pois[:, 2:4]
    r = oracle.solve_pois(ref, coef, cfg, pois[:, :2], p0, gradients=oracle.reference_gradient(ref),
                          roi=masked["roi"], masked=True)
    want = masked[name]
    assert (want[:, 14] == 0).sum() > 60 and (want[:, 14] == 2).sum() > 60   # both kinds of points present
    _check_variant(r, want, P_TOL, Q_TOL, 1e-9)


# ---- whole propagations (tests/golden/subset_propagation_256.npz) ---------------------------
PROPAGATION_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_propagation_256.npz")


@pytest.fixture(scope="module")
def propagation():
    d = np.load(PROPAGATION_FILE)
    return {k: d[k] for k in d.files}


@pytest.mark.parametrize("tag,opt,order", [("full", 0, 1), ("roi", 0, 1), ("fgn", 1, 1), ("icgn2", 0, 2)])
def test_oracle_heap_propagation_matches_golden(oracle, golden, propagation, tag, opt, order):
    """The oracle's reliability-guided propagation in the reference's heap order against an
    independent transcription of ReliabilityPropagation::propagate: the same points solved and
    kept, the same flags and iteration counts, and the kept results to FP64 agreement.  ICGN over
    the full grid and under a ROI, FGN and second-order ICGN over the full grid."""
    g = propagation
    degree, border, radius, max_iter, thr, spacing, max_znssd = g["settings"]
    cfg = oracle.default_config()
    cfg.subset_radius, cfg.max_iterations, cfg.convergence_threshold = int(radius), int(max_iter), float(thr)
    cfg.degree, cfg.border, cfg.optimizer, cfg.shape_order, cfg.criterion = int(degree), int(border), opt, order, 1
    cfg.propagation_spacing, cfg.propagation_max_znssd, cfg.propagation_mode = int(spacing), float(max_znssd), 1
    ref = golden["reference"].astype(np.float32)
    coef = oracle.prefilter(golden["deformed"].astype(np.float32), int(degree), int(border), True)
    seed = oracle.make_seed(*g["seed_xy"], list(g["seed_p"]), float(g["seed_correlation"]))
    roi = g.get(f"mask_{tag}")
    got = oracle.propagate(ref, coef, cfg, seed, roi=roi, gradients=oracle.reference_gradient(ref))
    kept, solves = g[f"counts_{tag}"]
    assert got["points_computed"] == kept and got["solves"] == solves
    assert kept > (500 if roi is None else 150)
    assert (roi is None) == (f"mask_{tag}" not in g)
    valid = g[f"valid_{tag}"]
    assert np.array_equal(got["valid"], valid)
    assert np.array_equal(got["status"][valid], g[f"status_{tag}"][valid])
    assert np.array_equal(got["iterations"][valid], g[f"iterations_{tag}"][valid])
    p = np.column_stack([got[k] for k in ("u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "d2u_dx2", "d2u_dxdy",
                                          "d2u_dy2", "d2v_dx2", "d2v_dxdy", "d2v_dy2")])
    assert np.max(np.abs(p[valid] - g[f"p_{tag}"][valid])) <= P_TOL
    assert np.max(np.abs(got["correlation"][valid] - g[f"correlation_{tag}"][valid])) <= 1e-9
    if order == 2:
        assert np.abs(g[f"p_{tag}"][valid, 6:]).max() > 1e-6   # the curvature terms are exercised
    step = int(spacing) + 1
    gh, gw = got["grid_shape"]
    assert np.array_equal(got["x"], (np.arange(gw * gh) % gw) * float(step))


# ---- seed selection (tests/golden/subset_seed_256.npz) --------------------------------------
SEED_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_seed_256.npz")


@pytest.fixture(scope="module")
def seed_golden():
    d = np.load(SEED_FILE)
    return {k: d[k] for k in d.files}


def _seed_config(g, make_default):
    (is_r, search, pyr_scale, pyr_ref, count, km_iters, limit, max_znssd, min_tex, min_norm, degree, border,
     radius, max_iter, thr) = g["settings"]
    cfg = make_default()
    cfg.is_subset_radius, cfg.is_search_radius, cfg.pyramid_enabled = int(is_r), int(search), 1
    cfg.pyramid_scale, cfg.pyramid_refinement_radius = int(pyr_scale), int(pyr_ref)
    cfg.seed_count, cfg.kmeans_iterations, cfg.kmeans_sample_limit = int(count), int(km_iters), int(limit)
    cfg.seed_max_znssd, cfg.min_texture_std, cfg.min_displacement_norm = float(max_znssd), float(min_tex), float(min_norm)
    cfg.degree, cfg.border, cfg.subset_radius = int(degree), int(border), int(radius)
    cfg.sp_enabled, cfg.sp_subset_radius, cfg.sp_max_iterations = 1, int(radius), int(max_iter)
    cfg.sp_convergence_threshold = float(thr)
    return cfg


@pytest.mark.parametrize("tag", ["full", "roi", "truncated"])
def test_oracle_seed_selection_matches_golden(oracle, golden, seed_golden, tag):
    """SeedSelector::select_best_seed against an independent transcription: the k-means candidate
    list, every candidate's integer search (displacement and ZNCC), and the chosen seed with its
    subpixel-refined parameters and ZNSSD.  "truncated": truncate_roi_subsets, so the candidate
    margin includes the search radius, and both the integer search and the refinement are masked
    by the ROI (17 of the 64 candidates' subsets cross its edge)."""
    g = seed_golden
    cfg = _seed_config(g, oracle.default_config)
    cfg.truncate_roi_subsets = int(tag == "truncated")
    ref, de = golden["reference"], golden["deformed"]
    roi = g.get(f"mask_{tag}")
    seed, cands = oracle.select_seed(ref, de, cfg, roi=roi)
    want = g[f"candidates_{tag}"]
    assert len(want) == cfg.seed_count and np.array_equal(cands, want.astype(np.float64))
    integer = g[f"integer_{tag}"]
    for (x, y), (u, v, z, found) in zip(want, integer):
        got = oracle.integer_search(ref, de, cfg, x, y, roi=roi if cfg.truncate_roi_subsets else None)
        assert (got is not None) == bool(found)
        if got is not None:
            assert (got[0], got[1]) == (u, v) and abs(got[2] - z) <= 1e-12
    best = int(g[f"best_{tag}"])
    assert best >= 0 and seed.found
    ev = g[f"evaluations_{tag}"][best]
    assert (seed.x, seed.y) == tuple(want[best].astype(np.float64))
    assert np.max(np.abs(np.array(list(seed.p)) - ev[:6])) <= P_TOL
    assert abs(seed.correlation - ev[6]) <= 1e-9


# ---- SubsetDIC::compute with truncated subsets (tests/golden/subset_truncated_256.npz) -------
TRUNCATED_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_truncated_256.npz")


@pytest.fixture(scope="module")
def truncated_golden():
    d = np.load(TRUNCATED_FILE)
    return {k: d[k] for k in d.files}


@pytest.mark.parametrize("tag", ["full", "roi"])
def test_oracle_truncated_compute_matches_golden(oracle, golden, truncated_golden, tag):
    """SubsetDIC::compute with truncate_roi_subsets against an independent transcription: mirror
    padding, seed selection and heap-order propagation with masked subsets on the padded images,
    the grid cropped to the image and shifted back.  Same points, flags and iteration counts;
    parameters to FP64 agreement; the seed in image coordinates."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    g = truncated_golden
    cfg = oracle.as_config(S.config_from_dict(G.WORKLOAD0_CONFIG))
    cfg.truncate_roi_subsets, cfg.propagation_mode = 1, 1
    roi = g.get(f"mask_{tag}")
    got = oracle.subset_compute(golden["reference"], golden["deformed"], cfg, roi=roi)
    kept, solves, pad = g[f"counts_{tag}"]
    assert pad == oracle.subset_padding(cfg)
    assert np.array_equal(got["x"], g[f"x_{tag}"]) and np.array_equal(got["y"], g[f"y_{tag}"])
    valid = g[f"valid_{tag}"]
    assert np.array_equal(got["valid"], valid) and valid.sum() == kept
    assert np.array_equal(got["iterations"][valid], g[f"iterations_{tag}"][valid])
    p = np.column_stack([got[k] for k in ("u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy")])
    assert np.max(np.abs(p[valid] - g[f"p_{tag}"][valid, :6])) <= P_TOL
    assert np.max(np.abs(got["correlation"][valid] - g[f"correlation_{tag}"][valid])) <= 1e-9
    seed = g[f"seed_{tag}"]
    assert (got["seed"].x, got["seed"].y) == (seed[0] - pad, seed[1] - pad)
    assert np.max(np.abs(np.array(list(got["seed"].p)) - seed[2:8])) <= P_TOL
    if tag == "full":   # points whose full subset would leave the image are solved
        edge = (got["x"] < 10) | (got["y"] < 10) | (got["x"] >= 246) | (got["y"] >= 246)
        assert valid[edge].sum() > 50


# ---- the quintic B-spline (tests/golden/subset_degree5_256.npz) -----------------------------
DEGREE5_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_degree5_256.npz")
DEGREE5 = [("icgn1_znssd", 0, 1, 1), ("fgn1_znssd", 1, 1, 1), ("icgn2_znssd", 0, 2, 1), ("fgn2_ssd", 1, 2, 0)]


@pytest.fixture(scope="module")
def degree5():
    d = np.load(DEGREE5_FILE)
    return {k: d[k] for k in d.files}


@pytest.mark.parametrize("name,opt,order,crit", DEGREE5)
def test_oracle_degree5_matches_golden(oracle, golden, degree5, name, opt, order, crit):
    """Degree 5, the reference's default spline: the coefficients and four solver routes."""
    cfg = _variant_config(degree5, oracle.default_config, opt, order, crit)
    assert cfg.degree == 5
    coef = oracle.prefilter(golden["deformed"].astype(np.float32), 5, cfg.border, True)
    crop = degree5["coef_crop"]
    assert np.max(np.abs(coef[:40, :40] - crop)) <= 1e-10 * max(1.0, np.abs(crop).max())
    ref = golden["reference"].astype(np.float32)
    pois = degree5["pois"]
    p0 = np.zeros((len(pois), 6))
    p0[:, :2] = pois[:, 2:4]
    r = oracle.solve_pois(ref, coef, cfg, pois[:, :2], p0, gradients=oracle.reference_gradient(ref))
    _check_variant(r, degree5[name], P_TOL, Q_TOL, 1e-9)
