"""GPU against the FP64 oracle at the benchmark's own size: the 2048 x 2048 uint8 speckle pair
(24000 blobs, sinusoidal field), radius 15, POI step 5 (410 x 410 = 168,100 grid points),
first-order ZNSSD ICGN, bicubic spline, threshold 1e-3, 20 iterations.  Both run the dataflow
visit order from the oracle's seed; the oracle spreads each dataflow diagonal over the host's
threads (the same result as one thread).

Tolerances.  FP64: the same flags, iteration counts and convergence flags on every point, u and v
to 1e-7 px, displacement gradients to 1e-7, ZNSSD to 1e-9.  FP32-mixed: flags identical on
>= 99.9 % of the points; of the jointly valid points >= 99.99 % within 1e-3 px in u and v and
within 1e-5 in ZNCC, >= 99.9 % within 1e-5 in each displacement gradient, p99 of |du|, |dv| below
1e-5 px.  (Measured on a GB300: flags identical on all points; 5 of 162,936 points beyond
1e-3 px, all iterates of solves that did not converge in 20 iterations or their children.)"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = ("u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy")


@pytest.fixture(scope="module")
def c2(oracle):
    import __graft_entry__ as G  # noqa: F401
    from traditional_dic_gb300 import synthetic
    import bench
    p = synthetic.workload(1)
    cfg = bench.oracle_config(oracle, bench.CONFIG, 2)
    seed, _ = oracle.select_seed(p.reference, p.deformed, cfg)
    assert seed.found
    coef = oracle.prefilter(p.deformed.astype(np.float32), 3, 3, True)
    want = oracle.propagate(p.reference, coef, cfg, seed, threads=os.cpu_count() or 1)
    return p, seed, want


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_c2_propagation_matches_oracle(gpu_ctx, c2, precision):
    from traditional_dic_gb300 import subset as S
    import bench
    p, oseed, want = c2
    cfg = S.config_from_dict(dict(bench.CONFIG, gpu={"precision": precision, "propagation": "dataflow"}))
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, precision=cfg.precision)
    got = S.propagate(gpu_ctx, pair, cfg, S.make_seed(oseed.x, oseed.y, list(oseed.p), oseed.correlation))
    pair.close()
    assert want["points_computed"] > 160000
    if precision == "fp64":
        assert got["points_computed"] == want["points_computed"]
        assert np.array_equal(got["valid"], want["valid"])
        assert np.array_equal(got["iterations"], want["iterations"])
        assert np.array_equal(got["converged"], want["converged"])
        ok = want["valid"]
        for k in PARAMS:
            assert np.max(np.abs(got[k][ok] - want[k][ok])) <= 1e-7, k
        assert np.max(np.abs(got["correlation"][ok] - want["correlation"][ok])) <= 1e-9
        return
    assert np.mean(got["valid"] == want["valid"]) >= 0.999
    both = got["valid"] & want["valid"]
    du, dv = np.abs(got["u"] - want["u"])[both], np.abs(got["v"] - want["v"])[both]
    assert np.mean((du <= 1e-3) & (dv <= 1e-3)) >= 0.9999
    assert np.quantile(du, 0.99) <= 1e-5 and np.quantile(dv, 0.99) <= 1e-5
    for k in PARAMS[2:]:
        assert np.mean(np.abs(got[k] - want[k])[both] <= 1e-5) >= 0.999, k
    assert np.mean(np.abs(got["zncc"] - want["zncc"])[both] <= 1e-5) >= 0.9999


def test_c2_integer_search_matches_oracle(oracle, gpu_ctx):
    """The integer search at the benchmark's size (one coarse pass over 2028 / 4 x 2028 / 4
    positions per candidate): every one of the oracle's 64 seed candidates, displacement exactly,
    FP64 ZNCC to 1e-12."""
    from traditional_dic_gb300 import subset as S, synthetic
    import bench
    p = synthetic.workload(1)
    ocfg = bench.oracle_config(oracle, bench.CONFIG, 2)
    _, cand = oracle.select_seed(p.reference, p.deformed, ocfg)
    assert len(cand) == 64
    xs = np.array([int(round(c[0])) for c in cand], np.int32)
    ys = np.array([int(round(c[1])) for c in cand], np.int32)
    cfg = S.config_from_dict(bench.CONFIG)
    pair = S.Pair(gpu_ctx, p.reference, p.deformed, degree=3, exact=False)
    got = S.integer_search(gpu_ctx, pair, cfg, xs, ys)
    pair.close()
    assert got["ok"].all()
    for i in range(len(xs)):
        want = oracle.integer_search(p.reference, p.deformed, ocfg, xs[i], ys[i])
        assert want is not None
        assert (got["u"][i], got["v"][i]) == (want[0], want[1]), i
        assert abs(got["zncc"][i] - want[2]) <= 1e-12, i
