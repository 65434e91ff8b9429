"""Least-squares strain and result files.  CPU: the numpy oracle of
compute_least_squares_strain_2d on exact fields and degenerate neighbourhoods, and the result
writers.  GPU: the device strain against the oracle."""
import csv
import json
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import strain_oracle as SO  # noqa: E402


def _grid(nx=12, ny=9, step=5.0):
    ys, xs = np.mgrid[0:ny, 0:nx].astype(np.float64) * step
    return np.column_stack([xs.ravel() + 3.0, ys.ravel() + 7.0])


def test_oracle_recovers_an_affine_field():
    pts = _grid()
    h = np.array([[0.01, -0.004], [0.003, 0.02]])
    disp = 0.7 + pts @ h.T
    r = SO.least_squares_strain_2d(pts, disp, radius=12.0, min_samples=6, green_lagrange=True)
    assert r["valid"].all()
    for k, want in (("du_dx", h[0, 0]), ("du_dy", h[0, 1]), ("dv_dx", h[1, 0]), ("dv_dy", h[1, 1])):
        assert np.allclose(r[k], want, atol=1e-12), k
    e = 0.5 * (h + h.T + h.T @ h)
    assert np.allclose(r["exx"], e[0, 0]) and np.allclose(r["eyy"], e[1, 1]) and np.allclose(r["exy"], e[0, 1])
    small = SO.least_squares_strain_2d(pts, disp, radius=12.0, green_lagrange=False)
    assert np.allclose(small["exy"], 0.5 * (h[0, 1] + h[1, 0]))
    # a centre point has the 5-px neighbours within 12 px: (2*2+1)^2 - 4 corners
    assert r["sample_count"][5 * 12 + 5] == 21


def test_oracle_degenerate_neighbourhoods():
    line = np.column_stack([np.arange(10.0) * 4.0, np.full(10, 2.0)])
    disp = np.column_stack([0.1 + 0.02 * line[:, 0], -0.3 + 0.0 * line[:, 0]])
    r = SO.least_squares_strain_2d(line, disp, radius=9.0, min_samples=3)
    inner = r["valid"]
    assert inner.any()
    assert np.allclose(r["du_dx"][inner], 0.02) and np.all(r["du_dy"][inner] == 0.0)  # basic solution
    few = SO.least_squares_strain_2d(line, disp, radius=3.0, min_samples=3)
    assert not few["valid"].any() and np.all(few["sample_count"] == 1)
    bad = disp.copy()
    bad[4, 0] = np.nan
    r = SO.least_squares_strain_2d(line, bad, radius=9.0, min_samples=3)
    assert not r["valid"][4] and r["sample_count"][4] == 0 and r["sample_count"][3] == 4


def test_result_writers(tmp_path, pkg):
    from traditional_dic_gb300 import results
    n = 7
    res = {k: np.linspace(-1, 1, n) for k in results.SUBSET_COLUMNS[:-1]}
    res["valid"] = np.array([1, 0, 1, 1, 0, 1, 1], bool)
    results.save_subset_csv(res, tmp_path / "d.csv")
    rows = list(csv.reader(open(tmp_path / "d.csv")))
    assert rows[0] == results.SUBSET_COLUMNS and len(rows) == n + 1
    assert float(rows[3][2]) == res["u"][2] and rows[2][-1] == "0"
    results.write_stats(res, tmp_path / "s.json")
    st = json.loads(open(tmp_path / "s.json").read())
    assert st["total_points"] == 7 and st["valid_points"] == 5 and "znssd_mean" in st
    assert st["u_mean"] == pytest.approx(res["u"][res["valid"]].mean())


def _python_csv(res, path):
    """The reference's writer loop (csv.writer, str() of each float, int valid) as the checker."""
    from traditional_dic_gb300 import results
    cols = [np.asarray(res[k]) for k in results.SUBSET_COLUMNS]
    with open(path, "w", newline="", encoding="utf-8") as f:
        w = csv.writer(f)
        w.writerow(results.SUBSET_COLUMNS)
        for i in range(len(cols[0])):
            w.writerow([float(c[i]) for c in cols[:-1]] + [int(cols[-1][i])])


def test_subset_csv_bytes_equal_csv_writer(tmp_path, pkg):
    """The library's CSV writer against csv.writer byte for byte: random doubles over every
    decimal exponent, the positional/scientific switches (1e-4 / 1e-5, 1e15 / 1e16), integers,
    signed zeros, NaN and infinities, denormals and the extremes, and an empty grid."""
    from traditional_dic_gb300 import results
    rng = np.random.default_rng(11)
    special = np.array([0.0, -0.0, 1.0, -1.0, 0.1, 1e-4, 9.999e-5, 1e-5, 1.5e-5, 123456789012345.0,
                        1e15, 9999999999999998.0, 1e16, 1.5e16, 1e22, 1e100, 5e-324, 2.2250738585072014e-308,
                        1.7976931348623157e308, np.nan, np.inf, -np.inf, 1234567.0, 0.30000000000000004,
                        100.0, 2.5, -3.75e-7, 6.02214076e23, 1 / 3, 2 / 3])
    n = 5000
    mant = rng.uniform(-10, 10, n) * 10.0 ** rng.integers(-30, 30, n)
    for k, name in enumerate(results.SUBSET_COLUMNS[:-1]):
        col = rng.permutation(np.concatenate([special, mant[: n - len(special)]]))
        if k == 0:
            col[:len(special)] = special
        res_k = col
        if name in ("x", "y"):
            res_k = np.where(rng.random(n) < 0.5, np.round(col), col)
        if k == 0:
            res = {}
        res[name] = res_k
    res["u"][: 64] = rng.standard_normal(64).astype(np.float32)  # float32 values widened to double
    res["valid"] = rng.random(n) < 0.7
    results.save_subset_csv(res, tmp_path / "native.csv")
    _python_csv(res, tmp_path / "python.csv")
    assert (tmp_path / "native.csv").read_bytes() == (tmp_path / "python.csv").read_bytes()
    empty = {k: np.zeros(0) for k in results.SUBSET_COLUMNS}
    results.save_subset_csv(empty, tmp_path / "e.csv")
    _python_csv(empty, tmp_path / "pe.csv")
    assert (tmp_path / "e.csv").read_bytes() == (tmp_path / "pe.csv").read_bytes()
    with pytest.raises(Exception, match="cannot open"):
        results.save_subset_csv(res, tmp_path / "missing_dir" / "x" / "..")


def _compare(got, want, tol=1e-9):
    assert np.array_equal(got.valid, want["valid"])
    assert np.array_equal(got.sample_count, want["sample_count"])
    v = want["valid"]
    for k in ("du_dx", "du_dy", "dv_dx", "dv_dy", "exx", "eyy", "exy"):
        assert np.allclose(got[k][v], want[k][v], rtol=0, atol=tol), k


@pytest.mark.gpu
def test_gpu_strain_matches_oracle_on_points(gpu_ctx):
    from traditional_dic_gb300 import postprocess as P
    rng = np.random.default_rng(5)
    pts = rng.uniform(0, 300, (4000, 2))
    disp = np.column_stack([0.5 + 0.003 * pts[:, 0] - 0.001 * pts[:, 1], -0.2 + 0.002 * pts[:, 1]])
    disp += rng.normal(0, 0.01, disp.shape)
    disp[::97] = np.nan
    for green in (True, False):
        got = P.compute_least_squares_strain_2d(pts, disp, 15.0, 6, green, context=gpu_ctx)
        _compare(got, SO.least_squares_strain_2d(pts, disp, 15.0, 6, green))
    line = np.column_stack([np.arange(20.0) * 3.0, np.full(20, 5.0)])
    ld = np.column_stack([0.02 * line[:, 0], 0.01 * line[:, 0]])
    _compare(P.compute_least_squares_strain_2d(line, ld, 7.0, 3, True, context=gpu_ctx),
             SO.least_squares_strain_2d(line, ld, 7.0, 3, True))
    with pytest.raises(Exception, match="radius must be positive"):
        P.compute_least_squares_strain_2d(pts, disp, 0.0, 6, context=gpu_ctx)


@pytest.mark.gpu
def test_gpu_strain_of_a_subset_result(gpu_ctx, workload0, tmp_path):
    import __graft_entry__ as G
    from traditional_dic_gb300 import postprocess as P, subset as S
    res = S.compute(workload0.reference, workload0.deformed, G.WORKLOAD0_CONFIG, context=gpu_ctx)
    v = res["valid"]
    pts = np.column_stack([res["x"][v], res["y"][v]])
    disp = np.column_stack([res["u"][v], res["v"][v]])
    got = P.compute_least_squares_strain_2d(pts, disp, 25.0, 6, True, context=gpu_ctx)
    _compare(got, SO.least_squares_strain_2d(pts, disp, 25.0, 6, True))
    # the imposed field: du/dx = 0.001, dv/dy = -0.0005
    assert abs(np.median(got.du_dx[got.valid]) - 0.001) < 2e-4
    assert abs(np.median(got.dv_dy[got.valid]) + 0.0005) < 2e-4
    P.save_least_squares_strain_csv(tmp_path / "strain.csv", pts, disp, radius=25.0, context=gpu_ctx)
    rows = list(csv.reader(open(tmp_path / "strain.csv")))
    assert rows[0][:3] == ["x", "y", "du_dx"] and len(rows) == len(pts) + 1


def test_oracle_matches_a_brute_force_transcription():
    """compute_least_squares_strain_2d (least_squares_strain.cpp:11-78) restated without buckets:
    every finite point's neighbours within the radius (inclusive) by brute force, the [1, dx, dy]
    fit by numpy's least squares, small and Green-Lagrange strains.  Scattered points, a quadratic
    field (the fit is not exact), points with NaN coordinates or displacements, and neighbourhoods
    below min_samples."""
    rng = np.random.default_rng(21)
    n = 400
    pts = rng.uniform(0, 120, (n, 2))
    pts[::37, 0] = np.nan
    disp = np.column_stack([0.3 + 0.01 * pts[:, 0] - 2e-4 * pts[:, 1] ** 2,
                            -0.2 + 3e-4 * pts[:, 0] * pts[:, 1] + 0.004 * pts[:, 1]])
    disp[5::41, 1] = np.nan
    radius, min_samples = 9.5, 6
    for gl in (True, False):
        got = SO.least_squares_strain_2d(pts, disp, radius, min_samples, gl)
        finite = np.all(np.isfinite(pts), axis=1) & np.all(np.isfinite(disp), axis=1)
        for i in range(n):
            if not finite[i]:
                assert got["sample_count"][i] == 0 and not got["valid"][i]
                continue
            d2 = np.sum((pts - pts[i]) ** 2, axis=1)
            ids = np.nonzero(finite & (d2 <= radius * radius))[0]
            assert got["sample_count"][i] == len(ids)
            if len(ids) < min_samples:
                assert not got["valid"][i]
                continue
            a = np.column_stack([np.ones(len(ids)), pts[ids, 0] - pts[i, 0], pts[ids, 1] - pts[i, 1]])
            assert np.linalg.matrix_rank(a) == 3
            au = np.linalg.lstsq(a, disp[ids, 0], rcond=None)[0]
            av = np.linalg.lstsq(a, disp[ids, 1], rcond=None)[0]
            h = np.array([[au[1], au[2]], [av[1], av[2]]])
            e = 0.5 * (h + h.T + h.T @ h) if gl else np.array([[h[0, 0], 0.5 * (h[0, 1] + h[1, 0])],
                                                             [0.5 * (h[0, 1] + h[1, 0]), h[1, 1]]])
            assert got["valid"][i]
            want = (h[0, 0], h[0, 1], h[1, 0], h[1, 1], e[0, 0], e[1, 1], e[0, 1])
            for k, w in zip(("du_dx", "du_dy", "dv_dx", "dv_dy", "exx", "eyy", "exy"), want):
                assert abs(got[k][i] - w) <= 1e-11, (i, k)
        assert got["valid"].sum() > 250 and (~got["valid"] & finite).sum() > 0
