"""Test oracle (test infrastructure only): a numpy restatement of the reference's least-squares
strain, dic::compute_least_squares_strain_2d (src/postprocess/least_squares_strain.cpp:11-78).
Buckets of side `radius` keyed by floor(coordinate / radius); per point the neighbours within
`radius` from the 3 x 3 surrounding buckets (bucket rows, then columns, then point index); the fit
[1, dx, dy] p = u solved as Eigen's ColPivHouseholderQR::solve does: QR with column pivoting, rank
from the pivots (|R_ii| > eps * min(m, 3) * |R_00|), the basic solution (zeros for the columns
beyond the rank)."""
import math

import numpy as np
import scipy.linalg

FIELDS = ("du_dx", "du_dy", "dv_dx", "dv_dy", "exx", "eyy", "exy", "sample_count", "valid")


def _solve_colpiv(a, b):
    q, r, perm = scipy.linalg.qr(a, mode="economic", pivoting=True)
    diag = np.abs(np.diag(r))
    if diag.size == 0 or diag[0] == 0.0:
        return np.zeros(a.shape[1])
    tol = np.finfo(np.float64).eps * min(a.shape) * diag[0]
    rank = int(np.sum(diag > tol))
    y = q.T @ b
    x = np.zeros(a.shape[1])
    x[perm[:rank]] = scipy.linalg.solve_triangular(r[:rank, :rank], y[:rank])
    return x


def least_squares_strain_2d(points, displacement, radius, min_samples=6, green_lagrange=True):
    pts = np.asarray(points, np.float64)
    dsp = np.asarray(displacement, np.float64)
    n = pts.shape[0]
    out = {k: np.zeros(n) for k in FIELDS[:7]}
    out["sample_count"] = np.zeros(n, np.int32)
    out["valid"] = np.zeros(n, bool)
    finite = np.all(np.isfinite(pts), axis=1) & np.all(np.isfinite(dsp), axis=1)
    buckets = {}
    for i in np.nonzero(finite)[0]:
        key = (math.floor(pts[i, 0] / radius), math.floor(pts[i, 1] / radius))
        buckets.setdefault(key, []).append(i)
    r2 = radius * radius
    for i in np.nonzero(finite)[0]:
        bx, by = math.floor(pts[i, 0] / radius), math.floor(pts[i, 1] / radius)
        ids = []
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                for j in buckets.get((bx + dx, by + dy), ()):
                    if np.sum((pts[j] - pts[i]) ** 2) <= r2:
                        ids.append(j)
        out["sample_count"][i] = len(ids)
        if len(ids) < min_samples:
            continue
        a = np.column_stack([np.ones(len(ids)), pts[ids, 0] - pts[i, 0], pts[ids, 1] - pts[i, 1]])
        au = _solve_colpiv(a, dsp[ids, 0])
        av = _solve_colpiv(a, dsp[ids, 1])
        if not (np.all(np.isfinite(au)) and np.all(np.isfinite(av))):
            continue
        h = np.array([[au[1], au[2]], [av[1], av[2]]])
        out["du_dx"][i], out["du_dy"][i], out["dv_dx"][i], out["dv_dy"][i] = h[0, 0], h[0, 1], h[1, 0], h[1, 1]
        if green_lagrange:
            e = 0.5 * (h + h.T + h.T @ h)
            out["exx"][i], out["eyy"][i], out["exy"][i] = e[0, 0], e[1, 1], e[0, 1]
        else:
            out["exx"][i], out["eyy"][i], out["exy"][i] = h[0, 0], h[1, 1], 0.5 * (h[0, 1] + h[1, 0])
        out["valid"][i] = True
    return out
