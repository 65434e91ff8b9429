"""Batched propagation (tdic_batch_*): several uneven image pairs in one persistent launch must
give, job by job, the results of the single-pair propagation in the same (dataflow) order."""
import numpy as np
import pytest

from conftest import small_speckle

pytestmark = pytest.mark.gpu

U_TOL = 1e-3       # px
FLAG_AGREE = 0.999
KEYS = ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "zncc", "valid", "converged",
        "iterations", "status")

# (shape, dtype, subset radius, POI step, field offsets)
JOBS = [((160, 200), np.uint8, 7, 3, (0.4, -0.3)),
        ((256, 256), np.uint16, 11, 5, (-1.2, 0.8)),
        ((300, 220), np.uint8, 15, 8, (2.1, 1.4)),
        ((192, 192), np.uint16, 11, 3, (0.0, -2.5)),
        ((240, 320), np.uint8, 7, 5, (-0.7, 0.2))]


def _config(S, radius, step):
    return S.config_from_dict({
        "subset": {"radius": radius},
        "optimization": {"max_iterations": 20, "convergence_threshold": 1e-3},
        "interpolation": {"degree": 3},
        "initialization": {"integer_search": {"subset_radius": 7, "search_radius": 8, "sift_enabled": False},
                           "subpixel_refinement": {"subset_radius": 7}},
        "seed_selection": {"seed_count": 16, "max_znssd": 0.5},
        "reliability_propagation": {"spacing": step - 1, "max_znssd": 0.5},
        "gpu": {"propagation": "dataflow"}})


@pytest.fixture(scope="module")
def batch_inputs(gpu_ctx):
    from traditional_dic_gb300 import subset as S
    pairs, cfgs, seeds, rois = [], [], [], []
    for k, (shape, dtype, radius, step, (u0, v0)) in enumerate(JOBS):
        sp = small_speckle(shape, n=int(shape[0] * shape[1] / 45), seed=11 + k, u0=u0, v0=v0, dtype=dtype)
        cfg = _config(S, radius, step)
        lazy = S.Pair(gpu_ctx, sp.reference, sp.deformed, degree=3, exact=False)
        seed = S.select_seed(gpu_ctx, lazy, sp.reference.astype(np.float32), cfg)
        assert seed.found, k
        pairs.append(S.Pair(gpu_ctx, sp.reference, sp.deformed, degree=3))
        cfgs.append(cfg)
        seeds.append(seed)
        roi = None
        if k == 2:  # a ROI with a hole away from the seed
            roi = np.ones(shape, bool)
            h, w = shape
            y0 = h // 8 if seed.y >= h // 2 else h // 2 + h // 8
            roi[y0:y0 + h // 5, : w // 3] = False
        rois.append(roi)
    return pairs, cfgs, seeds, rois


def _single(S, ctx, pair, cfg, seed, roi):
    return S.propagate(ctx, pair, cfg, seed, roi=roi)


def test_batch_matches_single_propagation(gpu_ctx, batch_inputs):
    from traditional_dic_gb300 import subset as S
    pairs, cfgs, seeds, rois = batch_inputs
    b = S.Batch(gpu_ctx, pairs, cfgs, seeds, rois)
    assert b.config() == (4, 3, "full")  # untuned: 4-warp groups, three per block, as the single path
    for _ in range(2):           # the second launch reuses (and re-initialises) the scratch
        b.launch()
        pc = b.finish()
        for j in range(len(pairs)):
            want = _single(S, gpu_ctx, pairs[j], cfgs[j], seeds[j], rois[j])
            got = b.outputs(j)
            assert pc[j] == want["points_computed"] and pc[j] > 1, j
            for k in KEYS:
                assert np.array_equal(got[k], want[k], equal_nan=True), (j, k)
    b.close()


def test_batch_device_outputs_to_csv(gpu_ctx, batch_inputs, tmp_path):
    """The subset CSV written straight from a job's device arrays equals the one written from
    its host copy, byte for byte."""
    from traditional_dic_gb300 import subset as S, results
    pairs, cfgs, seeds, rois = batch_inputs
    b = S.Batch(gpu_ctx, pairs, cfgs, seeds, rois)
    b.launch()
    b.finish()
    for j in (0, 2):
        gh, gw = b.grid_shapes[j]
        results.save_subset_csv_device(b.device_outputs(j), gh * gw, tmp_path / f"dev{j}.csv", context=gpu_ctx)
        results.save_subset_csv(b.outputs(j), tmp_path / f"host{j}.csv")
        assert (tmp_path / f"dev{j}.csv").read_bytes() == (tmp_path / f"host{j}.csv").read_bytes(), j
    b.close()


def test_batch_job_without_seed_keeps_defaults(gpu_ctx, batch_inputs):
    from traditional_dic_gb300 import subset as S, _lib as L
    pairs, cfgs, seeds, _ = batch_inputs
    none = L.Seed()  # found = 0
    b = S.Batch(gpu_ctx, pairs[:2], cfgs[:2], [seeds[0], none])
    b.launch()
    pc = b.finish()
    assert pc[0] > 1 and pc[1] == 0
    out = b.outputs(1)
    assert not out["valid"].any() and np.all(out["u"] == 0.0)
    b.close()


def test_batch_tuned_graph_replay(gpu_ctx, batch_inputs):
    import torch
    from traditional_dic_gb300 import subset as S
    pairs, cfgs, seeds, rois = batch_inputs
    b = S.Batch(gpu_ctx, pairs, cfgs, seeds, rois)
    assert b.tune()[:2] in ((4, 2), (4, 1), (8, 1), (4, 3))
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        b.launch(stream=torch.cuda.current_stream())
    for _ in range(2):
        graph.replay()
        torch.cuda.synchronize()
        pc = b.finish()
        for j in range(len(pairs)):
            want = _single(S, gpu_ctx, pairs[j], cfgs[j], seeds[j], rois[j])
            got = b.outputs(j)
            assert abs(int(pc[j]) - want["points_computed"]) <= max(1, want["points_computed"] // 1000), j
            assert np.mean(got["valid"] == want["valid"]) >= FLAG_AGREE
            both = got["valid"] & want["valid"]
            assert np.max(np.abs(got["u"][both] - want["u"][both])) <= U_TOL
            assert np.max(np.abs(got["v"][both] - want["v"][both])) <= U_TOL
    del graph
    b.close()
