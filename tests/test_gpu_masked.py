"""GPU parity of masked subsets (truncate_roi_subsets): SubsetSolver::solve_with_mask on every
route (icgn.cpp:629-818, 990-1154, 1364-1562, 1741-1912; forward_gauss_newton.cpp:401-604,
796-968, 1299-1522, 1741-1941) and SubsetDIC::compute over padded images (subset_dic.cpp:53-104),
through the C ABI.

Against the golden vectors of tests/golden/subset_masked_256.npz (an independent numpy
transcription) and the FP64 CPU oracle.  Tolerances: FP64 build 1e-7 px with identical statuses
and iteration counts; FP32-mixed 1e-3 px, 1e-5 in the displacement gradients, flags identical on
>= 99.9 % of points.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U_TOL = 1e-3
G_TOL = 1e-5
FLAG_AGREE = 0.999
MASKED = [("icgn1_znssd", 0, 1, 1), ("icgn2_ssd", 0, 2, 0), ("fgn1_ssd", 1, 1, 0), ("fgn2_znssd", 1, 2, 1)]
ALL_ROUTES = [(o, s, c) for o in (0, 1) for s in (1, 2) for c in (1, 0)]


@pytest.fixture(scope="module")
def masked():
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "subset_masked_256.npz"))
    return {k: d[k] for k in d.files}


def _cfg(S, **kw):
    c = S.config_from_dict({"interpolation": {"degree": kw.pop("degree", 3)}})
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("precision", [1, 0])
@pytest.mark.parametrize("name,opt,order,crit", MASKED)
def test_masked_routes_match_golden(gpu_ctx, masked, workload0, name, opt, order, crit, precision):
    from traditional_dic_gb300 import subset as S
    degree, border, radius, max_iter, thr = masked["settings"]
    cfg = _cfg(S, degree=int(degree), border=int(border), subset_radius=int(radius), max_iterations=int(max_iter),
               convergence_threshold=float(thr), optimizer=opt, shape_order=order, criterion=crit,
               precision=precision, truncate_roi_subsets=1)
    pair = S.Pair(gpu_ctx, workload0.reference, workload0.deformed, degree=int(degree), border=int(border),
                  precision=precision)
    pois = masked["pois"]
    p0 = np.zeros((len(pois), 6))
    p0[:, :2] = pois[:, 2:4]
    got = S.solve_pois(gpu_ctx, pair, cfg, pois[:, :2], p0, roi=masked["roi"], masked=True)
    want = masked[name]
    wp, wq = want[:, :6], want[:, 6:12]
    wit, wst = want[:, 13].astype(int), want[:, 14].astype(int)
    ok = wst == 0
    assert ok.sum() > 60 and (wst == 2).sum() > 60
    if precision == 1:
        assert np.array_equal(got["status"], wst)
        assert np.array_equal(got["iterations"][ok], wit[ok])
        assert np.max(np.abs(got["p"][ok] - wp[ok])) <= 1e-7
        assert np.max(np.abs(got["q"][ok] - wq[ok])) <= 1e-8
    else:
        assert np.mean(got["status"] == wst) >= FLAG_AGREE
        both = ok & (got["status"] == 0)
        assert np.max(np.abs(got["p"][both, :2] - wp[both, :2])) <= U_TOL
        assert np.max(np.abs(got["p"][both, 2:] - wp[both, 2:])) <= G_TOL
    pair.close()


@pytest.mark.parametrize("opt,order,crit", ALL_ROUTES)
def test_masked_routes_fp64_match_oracle(oracle, gpu_ctx, workload0, opt, order, crit):
    """Every route masked by an annulus with a gap, POIs along its edges, and a sample floor
    (min_valid_sample_ratio 0.7) that some edge points miss."""
    from traditional_dic_gb300 import subset as S
    p = workload0
    h, w = p.reference.shape
    yy, xx = np.mgrid[:h, :w]
    rr = np.hypot(xx - 128, yy - 128)
    roi = (rr > 30) & (rr < 110) & ~((xx > 120) & (xx < 136))
    rng = np.random.default_rng(5)
    xy = rng.uniform(5, 250, size=(160, 2)).round()
    u, v = p.field.uv(xy[:, 0], xy[:, 1])
    p0 = np.zeros((len(xy), 6))
    p0[:, 0], p0[:, 1] = np.round(2 * u) / 2, np.round(2 * v) / 2
    cfg = _cfg(S, degree=3, subset_radius=9, max_iterations=20, convergence_threshold=1e-4, optimizer=opt,
               shape_order=order, criterion=crit, precision=1, truncate_roi_subsets=1, min_valid_samples=12,
               min_valid_sample_ratio=0.7)
    ref = p.reference.astype(np.float32) / 255.0
    de = p.deformed.astype(np.float32) / 255.0
    pair = S.Pair(gpu_ctx, ref, de, degree=3, precision=1)
    got = S.solve_pois(gpu_ctx, pair, cfg, xy, p0, roi=roi, masked=True)
    coef = oracle.prefilter(de, 3, 3, True)
    want = oracle.solve_pois(ref, coef, oracle.as_config(cfg), xy, p0, gradients=oracle.reference_gradient(ref),
                             roi=roi, masked=True)
    assert np.array_equal(got["status"], want["status"])
    assert (want["status"] == 0).sum() > 40 and (want["status"] == 2).sum() > 20
    same_it = got["iterations"] == want["iterations"]
    assert same_it.mean() >= 0.99
    ok = same_it & (want["status"] == 0)
    assert np.max(np.abs(got["p"][ok] - want["p"][ok])) < 1e-7
    assert np.max(np.abs(got["q"][ok] - want["q"][ok])) < 1e-8
    pair.close()


@pytest.mark.parametrize("with_roi", [False, True])
@pytest.mark.parametrize("precision", [1, 0])
def test_truncated_compute_matches_oracle(oracle, gpu_ctx, workload0, precision, with_roi):
    """SubsetDIC::compute with truncate_roi_subsets: padded images, masked seed search and
    refinement, masked propagation, the grid cropped and shifted back; against the oracle's
    pipeline in the GPU's visit order."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    roi = None
    if with_roi:
        yy, xx = np.mgrid[:256, :256]
        roi = ((xx - 150) ** 2 + (yy - 120) ** 2) < 100 ** 2
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    cfg.truncate_roi_subsets = 1
    cfg.precision = precision
    got, seed = S.compute_config(p.reference, p.deformed, cfg, roi, return_seed=True)
    ocfg = oracle.as_config(cfg)
    ocfg.propagation_mode = 2
    want = oracle.subset_compute(p.reference, p.deformed, ocfg, roi=roi)
    pad = oracle.subset_padding(ocfg)
    gw, gh = oracle.truncated_grid_dims(256, 256, ocfg)
    assert len(want["x"]) == gw * gh and len(got["x"]) == gw * gh
    assert np.array_equal(got["x"], want["x"]) and np.array_equal(got["y"], want["y"])
    assert got["x"][0] == (-pad) % 10 and got["y"][0] == (-pad) % 10
    assert seed.found and want["seed"].found
    assert (seed.x, seed.y) == (want["seed"].x, want["seed"].y)
    assert np.mean(got["valid"] == want["valid"]) >= FLAG_AGREE
    both = got["valid"] & want["valid"]
    tol = 1e-7 if precision == 1 else U_TOL
    assert np.max(np.abs(got["u"][both] - want["u"][both])) <= tol
    assert np.max(np.abs(got["v"][both] - want["v"][both])) <= tol
    # points whose full subset would leave the image are solved with truncated subsets
    edge = (got["x"] < cfg.subset_radius) | (got["y"] < cfg.subset_radius)
    if not with_roi:
        assert got["valid"][edge].mean() > 0.5


def test_masked_batch_matches_single(gpu_ctx, workload0):
    """Masked subsets in the batched launch: a job with a ROI that has holes (one touches the
    seed's neighbourhood) and a job without a ROI each give tdic_propagate's masked result bit for
    bit, untuned and tuned; a batch mixing masked and plain jobs is refused."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    p = workload0
    _, seed = S.compute(p.reference, p.deformed, G.WORKLOAD0_CONFIG, context=gpu_ctx, return_seed=True)
    assert seed.found
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    cfg.truncate_roi_subsets = 1
    cfg.propagation_mode = S.PROPAGATION_MODES["dataflow"]
    h, w = p.reference.shape
    roi = np.ones((h, w), bool)
    sx, sy = int(round(seed.x)), int(round(seed.y))
    roi[max(0, sy - 30):sy - 12, max(0, sx - 40):sx + 40] = False   # a band just above the seed
    roi[h // 8: h // 4, w // 2: w // 2 + 30] = False
    rois = [roi, None]
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3)
    keys = ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "zncc", "valid", "converged",
            "iterations", "status")
    want = [S.propagate(gpu_ctx, pair, cfg, seed, roi=r) for r in rois]
    b = S.Batch(gpu_ctx, [pair, pair], [cfg, cfg], [seed, seed], rois)
    for tuned in (False, True):
        if tuned:
            b.tune()
        b.launch()
        pc = b.finish()
        for j in range(2):
            got = b.outputs(j)
            assert pc[j] == want[j]["points_computed"] and pc[j] > 1, j
            for k in keys:
                assert np.array_equal(got[k], want[j][k], equal_nan=True), (tuned, j, k)
    b.close()
    plain = S.config_from_dict(G.WORKLOAD0_CONFIG)
    plain.propagation_mode = S.PROPAGATION_MODES["dataflow"]
    with pytest.raises(Exception, match="masked"):
        S.Batch(gpu_ctx, [pair, pair], [cfg, plain], [seed, seed])
    pair.close()
