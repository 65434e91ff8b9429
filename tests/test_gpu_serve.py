"""Serving loop (continuous batching): every request's result equals subset.compute of the same
pair alone, whether it was batched with others or not."""
import time

import numpy as np
import pytest

from conftest import small_speckle

pytestmark = pytest.mark.gpu

# (shape, dtype, radius, step, field offsets)
REQUESTS = [((180, 200), np.uint8, 7, 3, (0.4, -0.3)),
            ((256, 256), np.uint16, 11, 5, (-1.2, 0.8)),
            ((220, 300), np.uint8, 15, 8, (2.1, 1.4)),
            ((180, 200), np.uint16, 11, 3, (0.0, -2.5)),
            ((256, 256), np.uint8, 7, 5, (-0.7, 0.2)),
            ((200, 240), np.uint8, 15, 5, (1.5, -1.0)),
            ((180, 200), np.uint8, 7, 8, (0.3, 0.3)),
            ((256, 256), np.uint16, 11, 3, (-2.0, 1.1))]


def _config(radius, step, sift=False):
    return {"subset": {"radius": radius},
            "optimization": {"max_iterations": 20, "convergence_threshold": 1e-3},
            "interpolation": {"degree": 3},
            "initialization": {"integer_search": {"subset_radius": 7, "search_radius": 8, "sift_enabled": sift},
                               "subpixel_refinement": {"subset_radius": 7}},
            "seed_selection": {"seed_count": 16, "max_znssd": 0.5},
            "reliability_propagation": {"spacing": step - 1, "max_znssd": 0.5},
            "gpu": {"propagation": "dataflow"}}


def test_served_results_equal_alone(gpu_ctx):
    from traditional_dic_gb300 import serve, subset as S
    work = []
    for k, (shape, dtype, radius, step, (u0, v0)) in enumerate(REQUESTS):
        p = small_speckle(shape, n=int(shape[0] * shape[1] / 45), seed=40 + k, u0=u0, v0=v0, dtype=dtype)
        work.append((p.reference, p.deformed, _config(radius, step)))
    # a request without a seed (SIFT prior without OpenCV): the reference's empty result
    work.append((work[0][0], work[0][1], _config(7, 3, sift=True)))
    alone = [S.compute(r, d, c, context=gpu_ctx) for r, d, c in work]
    with serve.Server(gpu_ctx) as srv:
        reqs = [srv.submit(r, d, c) for r, d, c in work[:4]]
        time.sleep(0.003)                       # the rest arrive while the first ones are served
        reqs += [srv.submit(r, d, c) for r, d, c in work[4:]]
        served = [q.wait(300) for q in reqs]
        sizes = list(srv.batches)
    assert sum(sizes) == len(work) - 1          # the seedless request finishes without a batch
    assert max(sizes) > 1                       # requests shared a launch
    for k, (got, want) in enumerate(zip(served, alone)):
        assert set(got) == set(want), k
        for key in want:
            assert np.array_equal(got[key], want[key], equal_nan=True), (k, key)
    assert len(served[-1]["x"]) == 0
    assert all(q.latency > 0 for q in reqs)


def test_served_masked_requests_equal_alone(gpu_ctx):
    """Masked subsets (truncate_roi_subsets, a full Config structure) through the serving loop:
    tdic_subset_prepare pads the pair as tdic_subset_compute does, the batch propagates it with the
    padded ROI and the loop crops the grid back; every result equals subset.compute_config of
    the same request alone, bit for bit, with plain requests served beside them."""
    from traditional_dic_gb300 import serve, subset as S
    work = []
    for k, (shape, dtype, radius, step, (u0, v0)) in enumerate(REQUESTS[:5]):
        p = small_speckle(shape, n=int(shape[0] * shape[1] / 45), seed=60 + k, u0=u0, v0=v0, dtype=dtype)
        cfg = S.config_from_dict(_config(radius, step))
        cfg.truncate_roi_subsets = 1
        h, w = shape
        roi = None
        if k % 2 == 0:   # a hole right of the centre, and a corner cut off
            roi = np.ones(shape, bool)
            roi[h // 3: h // 3 + h // 6, w // 2 + 10: w // 2 + 10 + w // 5] = False
            roi[: h // 6, : w // 6] = False
        work.append((p.reference, p.deformed, cfg, roi))
    plain = small_speckle(REQUESTS[1][0], n=1100, seed=70, dtype=np.uint16)
    work.insert(2, (plain.reference, plain.deformed, _config(11, 5), None))   # a plain request between them

    def alone(r, d, c, roi):
        if isinstance(c, dict):
            return S.compute(r, d, c, roi, context=gpu_ctx)
        return S.compute_config(r, d, c, roi, context=gpu_ctx)

    want = [alone(*w_) for w_ in work]
    # the prepared pair is the padded one, its seed in padded coordinates
    r0, d0, c0, roi0 = work[0]
    _, seed0 = S.compute_config(r0, d0, c0, roi0, context=gpu_ctx, return_seed=True)
    pair, seed = S.prepare(gpu_ctx, r0, d0, c0, roi=roi0)
    pad = S.padding(c0)
    assert pad > 0 and (pair.height, pair.width) == (r0.shape[0] + 2 * pad, r0.shape[1] + 2 * pad)
    assert seed.found and (seed.x - pad, seed.y - pad) == (seed0.x, seed0.y)
    pair.close()
    with serve.Server(gpu_ctx) as srv:
        reqs = [srv.submit(r, d, c, roi) for r, d, c, roi in work]
        served = [q.wait(300) for q in reqs]
        sizes = list(srv.batches)
    assert sum(sizes) == len(work) and max(sizes) > 1
    for k, (got, exp) in enumerate(zip(served, want)):
        assert len(exp["x"]) > 0, k
        assert set(got) >= set(S.RESULT_KEYS + S.EXTRA_KEYS), k
        for key in S.RESULT_KEYS + S.EXTRA_KEYS:
            assert np.array_equal(got[key], exp[key], equal_nan=True), (k, key)
