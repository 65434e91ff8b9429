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
