"""Generate tests/golden/subset_icgn_256.npz: golden vectors for the subset-DIC path from an
independent numpy restatement of the reference (not the C++ oracle), so that the oracle and the
GPU path are both held to a second transcription.

Restated, from the reference sources:
  * B-spline coefficients (src/interpolation/bspline.cpp:177-244, 369-392): half-sample symmetric
    padding by `border`, then each row and each column deconvolved by the sampled B-spline kernel
    with a periodic FFT (numpy.fft here, kissfft there);
  * spline value (bspline.cpp:96-113, 320-367, 394-424, 458-474): the local polynomial block
    qk * C * qk^T of the coefficient neighbourhood, evaluated at (dx, dy);
  * first-order ZNSSD ICGN (src/subset/solver/icgn.cpp:446-627, update :83-120) with the reference
    gradients of the propagation (central differences on raw pixels,
    src/subset/seed/reliability_propagation.cpp:84-112); the 6 x 6 system is solved with
    numpy.linalg.solve (the reference factorises with LDLT: same solution for the positive
    definite Hessians of these points).

Input: the seeded 256 x 256 uint8 speckle pair of the small workload (stored in the file).  POIs:
a grid of subset centres (and one too close to the border) with initial guesses from the imposed
field rounded to 0.5 px and zero gradients.

Run from the repository root:  python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "subset_icgn_256.npz")

DEGREE, BORDER, RADIUS, MAX_ITER, THRESHOLD = 3, 3, 10, 20, 1e-3
EPS = 1e-12


def basis(x, r, d):
    if r < 0 or r > d:
        return 0.0
    fac = math.factorial(d) // math.factorial(d - r)
    s = 0.0
    for k in range(d + 2):
        shift = (d + 1) / 2.0 - k
        xx = x + shift
        s += (-1.0) ** k * math.comb(d + 1, k) * fac * (xx ** (d - r) if xx > 0 else 0.0)
    return s / math.factorial(d)


def qk_matrix(d):
    n, off = d + 1, d // 2
    return np.array([[(-1.0) ** r * basis(-off + c, r, d) / math.factorial(r) for c in range(n)] for r in range(n)])


def coefficients(image, d, border):
    h, w = image.shape
    ys = np.arange(-border, h + border)
    xs = np.arange(-border, w + border)

    def sym(v, size):
        p = 2 * size
        v = np.mod(v, p)
        return np.where(v < size, v, p - 1 - v)

    padded = image.astype(np.float64)[sym(ys, h)][:, sym(xs, w)]

    def kernel(length):
        k = np.zeros(length)
        k[0] = basis(0.0, 0, d)
        for o in range(1, d // 2 + 1):
            k[o] = k[length - o] = basis(float(o), 0, d)
        return k

    kr = np.fft.fft(kernel(padded.shape[1]))
    rows = np.real(np.fft.ifft(np.fft.fft(padded, axis=1) / kr[None, :], axis=1))
    kc = np.fft.fft(kernel(padded.shape[0]))
    return np.real(np.fft.ifft(np.fft.fft(rows, axis=0) / kc[:, None], axis=0))


def spline_values(coef, qk, xs, ys, w, h, d, border):
    off = d // 2
    ix = np.clip(np.floor(xs).astype(int), 0, w - 1)
    iy = np.clip(np.floor(ys).astype(int), 0, h - 1)
    dx, dy = xs - ix, ys - iy
    n = d + 1
    rr = np.clip(iy[:, None] + border - off + np.arange(n)[None, :], 0, coef.shape[0] - 1)
    cc = np.clip(ix[:, None] + border - off + np.arange(n)[None, :], 0, coef.shape[1] - 1)
    blocks = coef[rr[:, :, None], cc[:, None, :]]                      # (m, n, n): rows y, cols x
    poly = np.einsum("ra,mab,cb->mrc", qk, blocks, qk)
    ypow = dy[:, None] ** np.arange(n)[None, :]
    xpow = dx[:, None] ** np.arange(n)[None, :]
    return np.einsum("mrc,mr,mc->m", poly, ypow, xpow)


def ic_update(p, dp):
    du, dv, dudx, dudy, dvdx, dvdy = p
    d0, d1, d2, d3, d4, d5 = dp
    den = d2 + d5 + d2 * d5 - d3 * d4 + 1.0
    if abs(den) <= EPS:
        return np.full(6, np.nan)
    return np.array([
        du - ((dudx + 1.0) * (d0 + d0 * d5 - d1 * d3)) / den - (dudy * (d1 - d0 * d4 + d1 * d2)) / den,
        dv - ((dvdy + 1.0) * (d1 - d0 * d4 + d1 * d2)) / den - (dvdx * (d0 + d0 * d5 - d1 * d3)) / den,
        ((d5 + 1.0) * (dudx + 1.0)) / den - (d4 * dudy) / den - 1.0,
        (dudy * (d2 + 1.0)) / den - (d3 * (dudx + 1.0)) / den,
        (dvdx * (d5 + 1.0)) / den - (d4 * (dvdy + 1.0)) / den,
        ((d2 + 1.0) * (dvdy + 1.0)) / den - (d3 * dvdx) / den - 1.0])


def icgn(ref, coef, qk, px, py, p0):
    """(p[6], correlation, iterations, status, converged) of one POI; status: 0 success,
    1 not converged, 2 invalid input, 3 numerical failure."""
    h, w = ref.shape
    cx, cy = int(np.round(px)), int(np.round(py))
    r = RADIUS
    p = np.array([p0[0], p0[1], 0.0, 0.0, 0.0, 0.0])
    if cx - r < 0 or cy - r < 0 or cx + r >= w or cy + r >= h:
        return p, np.nan, 0, 2, False
    off = np.array([(dx, dy) for dy in range(-r, r + 1) for dx in range(-r, r + 1) if dx * dx + dy * dy <= r * r],
                   dtype=np.float64)
    lx, ly = off[:, 0], off[:, 1]
    xs, ys = cx + off[:, 0].astype(int), cy + off[:, 1].astype(int)
    f = ref[ys, xs].astype(np.float64)
    xm, xp = np.maximum(0, xs - 1), np.minimum(w - 1, xs + 1)
    ym, yp = np.maximum(0, ys - 1), np.minimum(h - 1, ys + 1)
    gx = (ref[ys, xp].astype(np.float64) - ref[ys, xm]) / np.maximum(1, xp - xm)
    gy = (ref[yp, xs].astype(np.float64) - ref[ym, xs]) / np.maximum(1, yp - ym)
    sd = np.column_stack([gx, gy, gx * lx, gx * ly, gy * lx, gy * ly])
    fm = f.mean()
    fn = math.sqrt(np.sum((f - fm) ** 2))
    if fn <= EPS:
        return p, np.inf, 0, 3, False
    fhat = (f - fm) / fn
    hess = sd.T @ sd * (2.0 / (fn * fn))
    corr, converged, it = np.inf, False, 0
    for it in range(1, MAX_ITER + 1):
        wx = cx + lx + p[0] + p[2] * lx + p[3] * ly
        wy = cy + ly + p[1] + p[4] * lx + p[5] * ly
        if np.any((wx < 0) | (wy < 0) | (wx > w - 1) | (wy > h - 1)):
            return p, corr, it, 2, False
        g = spline_values(coef, qk, wx, wy, w, h, DEGREE, BORDER)
        gm = g.mean()
        gn = math.sqrt(np.sum((g - gm) ** 2))
        if gn <= EPS:
            return p, corr, it, 3, False
        diff = fhat - (g - gm) / gn
        grad = (diff @ sd) * (2.0 / fn)
        corr = float(diff @ diff)
        dp = -np.linalg.solve(hess, grad)
        if not np.all(np.isfinite(dp)):
            return p, corr, it, 3, False
        p = ic_update(p, dp)
        if not np.all(np.isfinite(p)):
            return p, corr, it, 3, False
        if np.linalg.norm(dp) < THRESHOLD:
            converged = True
            break
    if not converged and math.isfinite(corr):
        converged = True
    return p, corr, it, 0 if converged else 1, converged


def main():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as G
    G.load_package()
    from traditional_dic_gb300 import synthetic
    pair = synthetic.workload(0)
    ref, de = pair.reference, pair.deformed
    h, w = ref.shape
    coef = coefficients(de, DEGREE, BORDER)
    qk = qk_matrix(DEGREE)
    pts = [(x, y) for y in range(20, 240, 22) for x in range(20, 240, 22)] + [(5.0, 128.0)]
    pois, res = [], []
    for x, y in pts:
        u, v = pair.field.uv(np.float64(x), np.float64(y))
        p0 = (round(2 * float(u)) / 2.0, round(2 * float(v)) / 2.0)
        p, corr, iters, status, conv = icgn(ref, coef, qk, x, y, p0)
        pois.append((x, y, p0[0], p0[1]))
        res.append(np.concatenate([p, [corr, iters, status, float(conv)]]))
    np.savez_compressed(OUT, reference=ref, deformed=de, coef_crop=coef[:40, :40],
                        pois=np.array(pois, np.float64), results=np.array(res, np.float64),
                        settings=np.array([DEGREE, BORDER, RADIUS, MAX_ITER, THRESHOLD]))
    print(f"wrote {OUT}: {len(pois)} POIs, {int(sum(r[9] for r in res))} converged")


if __name__ == "__main__":
    main()
