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

tests/golden/subset_variants_256.npz holds the other solver routes on the same POIs, for the
small workload's pair (affine field) and for a 256 x 256 pair with a Gaussian bump (curvature):
  * first-order SSD ICGN (icgn.cpp:832-988): raw residual f - g, Hessian and gradient unscaled;
  * second-order ZNSSD / SSD ICGN (icgn.cpp:142-357, 1168-1362, 1576-1739): 12 parameters, update
    through the 6 x 6 warp matrix G'(p) G'(dp)^-1 P^-1 (numpy.linalg.inv; additive update when
    G'(dp) is rank deficient);
  * FGN (forward_gauss_newton.cpp:622-794, 986-1053, 1069-1297, 1540-1739): SD from the spline
    gradient (bspline.cpp:115-151, 476-500) through dW/dz, step caps 0.5 (ZNSSD) / 0.35 (SSD),
    the first-order SSD route converging on the norm before the cap, and the second-order routes
    with the 1e-4 * max(diag H) damping term.

tests/golden/subset_masked_256.npz holds masked subsets (solve_with_mask, icgn.cpp:629-818 and
siblings; forward_gauss_newton.cpp:401-604, 796-968, 1299-1522, 1741-1941) over a disc ROI, with
POIs inside, on and outside its edge and at the image border: samples outside the image or the
ROI are dropped, the centre must be a ROI pixel (no margin check), at least max(6 or 12,
min_valid_samples = 12, ceil(0.5 * full circle)) samples are needed; the masked FGN routes cap the
step at 0.5 (first-order ZNSSD), 0.35 (SSD) and 0.3 (second-order ZNSSD, no damping term,
convergence on the norm before the cap).

tests/golden/subset_propagation_256.npz holds whole propagations over the small workload's grid
(ReliabilityPropagation::propagate, src/subset/seed/reliability_propagation.cpp:130-394) with the
first-order ZNSSD ICGN above, without and with a ROI, and over the full grid with the FGN and with
the second-order ICGN (the guesses carry the six first-order parameters): grid ceil(W/s) x ceil(H/s) for s = spacing
+ 1; the seed rounded (std::round), moved to the nearest grid point (llround, clamped) and solved
there again; a min-heap on ZNSSD; 4-neighbours up, right, down, left; ROI and margin admission;
the guess extrapolated with the parent's displacement gradients; strict acceptance (valid,
Success, ZNSSD < propagation_max_znssd, |guess - result| < s in u and v, all finite).

tests/golden/subset_seed_256.npz holds seed selections on the small workload's pair: without a ROI,
with a ROI, and with truncated subsets under a notched ROI, where the candidate margin adds the search
radius and the integer search (integer_search.cpp:447-545) and the refinement are masked
(SeedSelector::select_best_seed and generate_candidates,
src/subset/seed/seed_selector.cpp:146-317, 370-437): candidate pixels inside the ROI and the subset
margin, a deterministic sample of at most kmeans_sample_limit of them (llround of i * step), seed_count
k-means centres initialised the same way and moved kmeans_iterations times (nearest centre, lowest
index on ties), each centre rounded and checked for ROI, margin and texture (the population standard
deviation of the square window); then per candidate the integer search
(src/initialization/integer_search.cpp:129-280, 333-432: a coarse scan of the whole image at
pyramid_scale on the coarse circle, a refinement +-max(pyramid_refinement_radius, ceil(1.5 r)), a
local scan +-search_radius, the local winner kept when within 0.02 ZNCC) and the subpixel ICGN on the
clamp-padded raw deformed image (subset_initializer.cpp:152-204, bspline.cpp:302-318, 369-392), and
the best candidate by ZNSSD (1e-9 tolerance, then the larger displacement).

tests/golden/subset_degree5_256.npz holds the quintic spline (degree 5, the reference's default):
coefficients and the first-order ZNSSD ICGN and FGN, second-order ZNSSD ICGN and second-order SSD
FGN on the POIs above.

tests/golden/subset_truncated_256.npz holds SubsetDIC::compute with truncate_roi_subsets
(subset_dic.cpp:39-105, padding.cpp:11-90): both images mirror-padded and the ROI zero-padded by
recommended_subset_padding, the seed selected and the grid propagated (heap order, masked subsets) on
the padded images, and the grid points inside the original image returned shifted back.  The generator asserts
that no decision rests on a near tie, so its numpy summation order cannot change the result.

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


def spline_gradients(coef, qk, xs, ys, w, h, d, border):
    """d/dx and d/dy of the spline at (xs, ys): bspline.cpp:115-151 through the local block."""
    off = d // 2
    ix = np.clip(np.floor(xs).astype(int), 0, w - 1)
    iy = np.clip(np.floor(ys).astype(int), 0, h - 1)
    dx, dy = xs - ix, ys - iy
    n = d + 1
    rr = np.clip(iy[:, None] + border - off + np.arange(n)[None, :], 0, coef.shape[0] - 1)
    cc = np.clip(ix[:, None] + border - off + np.arange(n)[None, :], 0, coef.shape[1] - 1)
    blocks = coef[rr[:, :, None], cc[:, None, :]]
    poly = np.einsum("ra,mab,cb->mrc", qk, blocks, qk)
    k = np.arange(n)
    ypow = dy[:, None] ** k[None, :]
    xpow = dx[:, None] ** k[None, :]
    dxpow = np.where(k[None, :] >= 1, k[None, :] * dx[:, None] ** np.maximum(k - 1, 0)[None, :], 0.0)
    dypow = np.where(k[None, :] >= 1, k[None, :] * dy[:, None] ** np.maximum(k - 1, 0)[None, :], 0.0)
    return (np.einsum("mrc,mr,mc->m", poly, ypow, dxpow), np.einsum("mrc,mr,mc->m", poly, dypow, xpow))


def warp_matrix(p):
    u, v, ux, uy, vx, vy, uxx, uxy, uyy, vxx, vxy, vyy = p
    return np.array([
        [u, 1 + ux, uy, 0.5 * uxx, uxy, 0.5 * uyy],
        [v, vx, 1 + vy, 0.5 * vxx, vxy, 0.5 * vyy],
        [1, 0, 0, 0, 0, 0],
        [u * u, 2 * u * (1 + ux), 2 * u * uy, 1 + 2 * ux + ux * ux + u * uxx, 2 * (uy + ux * uy + u * uxy),
         uy * uy + u * uyy],
        [u * v, v + u * vx + v * ux, u + u * vy + v * uy, vx + ux * vx + 0.5 * (u * vxx + v * uxx),
         1 + vy + ux + ux * vy + uy * vx + u * vxy + v * uxy, uy + uy * vy + 0.5 * (u * vyy + v * uyy)],
        [v * v, 2 * v * vx, 2 * v * (1 + vy), vx * vx + v * vxx, 2 * (vx + vx * vy + v * vxy),
         1 + 2 * vy + vy * vy + v * vyy]])


def ic_update2(p, dp):
    gd = warp_matrix(dp)
    sv = np.linalg.svd(gd, compute_uv=False)
    if np.sum(sv > sv[0] * 6 * np.finfo(float).eps) < 6:
        return p - dp
    x = warp_matrix(p) @ np.linalg.inv(gd)
    n = x[:, [2, 0, 1, 3, 4, 5]]
    return np.array([n[0, 0], n[1, 0], n[0, 1] - 1, n[0, 2], n[1, 1], n[1, 2] - 1,
                     2 * n[0, 3], n[0, 4], 2 * n[0, 5], 2 * n[1, 3], n[1, 4], 2 * n[1, 5]])


def compose1(p, dp):
    return np.array([dp[0] + p[0] + p[2] * dp[0] + p[3] * dp[1], dp[1] + p[1] + p[4] * dp[0] + p[5] * dp[1],
                     dp[2] + p[2] * (1 + dp[2]) + p[3] * dp[4], dp[3] + p[2] * dp[3] + p[3] * (1 + dp[5]),
                     dp[4] + p[4] * (1 + dp[2]) + p[5] * dp[4], dp[5] + p[4] * dp[3] + p[5] * (1 + dp[5])])


def compose2(p, dp):
    q = np.empty(12)
    q[:6] = compose1(p[:6], dp[:6])
    q[2] += p[6] * dp[0] + p[7] * dp[1]
    q[3] += p[7] * dp[0] + p[8] * dp[1]
    q[4] += p[9] * dp[0] + p[10] * dp[1]
    q[5] += p[10] * dp[0] + p[11] * dp[1]
    q[6] = dp[6] + p[2] * dp[6] + p[3] * dp[9] + p[6] * (1 + 2 * dp[2]) + 2 * p[7] * dp[4]
    q[7] = dp[7] + p[2] * dp[7] + p[3] * dp[10] + p[6] * dp[3] + p[7] * (1 + dp[2] + dp[5]) + p[8] * dp[4]
    q[8] = dp[8] + p[2] * dp[8] + p[3] * dp[11] + p[7] * dp[3] + p[8] * (1 + 2 * dp[5])
    q[9] = dp[9] + p[4] * dp[6] + p[5] * dp[9] + p[9] * (1 + 2 * dp[2]) + 2 * p[10] * dp[4]
    q[10] = dp[10] + p[4] * dp[7] + p[5] * dp[10] + p[9] * dp[3] + p[10] * (1 + dp[2] + dp[5]) + p[11] * dp[4]
    q[11] = dp[11] + p[4] * dp[8] + p[5] * dp[11] + p[10] * dp[3] + p[11] * (1 + 2 * dp[5])
    return q


def shape_terms(lx, ly, order):
    m = [np.ones_like(lx), lx, ly]
    if order == 2:
        m += [lx * lx * 0.5, lx * ly, ly * ly * 0.5]
    return m


def sd_rows(a, b, lx, ly, order):
    m = shape_terms(lx, ly, order)
    cols = [a * m[0], b * m[0], a * m[1], a * m[2], b * m[1], b * m[2]]
    if order == 2:
        cols += [a * m[3], a * m[4], a * m[5], b * m[3], b * m[4], b * m[5]]
    return np.column_stack(cols)


def solve_variant(ref, coef, qk, px, py, p0, optimizer, order, ssd, roi=None, degree=DEGREE):
    """(p[12], correlation, iterations, status, converged) of one POI on one solver route;
    roi: the masked route over that mask."""
    h, w = ref.shape
    npar = 6 * order
    cx, cy = int(np.round(px)), int(np.round(py))
    r = RADIUS
    p = np.zeros(npar)
    p[:len(p0)] = p0
    out = lambda st, corr, it, conv: (np.concatenate([p[:6], p[6:], np.zeros(12 - npar)]), corr, it, st, conv)
    masked = roi is not None
    if masked:
        if not (0 <= cx < w and 0 <= cy < h) or not roi[cy, cx]:
            return out(2, np.nan, 0, False)
    elif cx - r < 0 or cy - r < 0 or cx + r >= w or cy + r >= h:
        return out(2, np.nan, 0, False)
    off = np.array([(dx, dy) for dy in range(-r, r + 1) for dx in range(-r, r + 1) if dx * dx + dy * dy <= r * r],
                   dtype=np.float64)
    full = len(off)
    if masked:
        xx, yy = cx + off[:, 0].astype(int), cy + off[:, 1].astype(int)
        inside = (xx >= 0) & (yy >= 0) & (xx < w) & (yy < h)
        keep = inside.copy()
        keep[inside] = roi[yy[inside], xx[inside]]
        off = off[keep]
        if len(off) < max(npar, 12, int(math.ceil(0.5 * full))):
            return out(2, np.nan, 0, False)
    lx, ly = off[:, 0], off[:, 1]
    xs, ys = cx + off[:, 0].astype(int), cy + off[:, 1].astype(int)
    f = ref[ys, xs].astype(np.float64)
    fn = 1.0
    if not ssd:
        fm = f.mean()
        fn = math.sqrt(np.sum((f - fm) ** 2))
        if fn <= EPS:
            return out(3, np.inf, 0, False)
        fhat = (f - fm) / fn
    if optimizer == 0:
        xm, xp = np.maximum(0, xs - 1), np.minimum(w - 1, xs + 1)
        ym, yp = np.maximum(0, ys - 1), np.minimum(h - 1, ys + 1)
        gx = (ref[ys, xp].astype(np.float64) - ref[ys, xm]) / np.maximum(1, xp - xm)
        gy = (ref[yp, xs].astype(np.float64) - ref[ym, xs]) / np.maximum(1, yp - ym)
        sd = sd_rows(gx, gy, lx, ly, order)
        hess = sd.T @ sd * (1.0 if ssd else 2.0 / (fn * fn))
    cap = 0.35 if ssd else (0.3 if masked and order == 2 else 0.5)
    test_capped = (not (order == 2 and not ssd)) if masked else (not (order == 1 and ssd))
    damping = order == 2 and (not masked or ssd)
    corr, converged, it = np.inf, False, 0
    for it in range(1, MAX_ITER + 1):
        m = shape_terms(lx, ly, order)
        wx = cx + lx + p[0] + p[2] * lx + p[3] * ly
        wy = cy + ly + p[1] + p[4] * lx + p[5] * ly
        if order == 2:
            wx = wx + p[6] * m[3] + p[7] * m[4] + p[8] * m[5]
            wy = wy + p[9] * m[3] + p[10] * m[4] + p[11] * m[5]
        if np.any((wx < 0) | (wy < 0) | (wx > w - 1) | (wy > h - 1)):
            return out(2, corr, it, False)
        g = spline_values(coef, qk, wx, wy, w, h, degree, BORDER)
        if ssd:
            diff = f - g
        else:
            gm = g.mean()
            gn = math.sqrt(np.sum((g - gm) ** 2))
            if gn <= EPS:
                return out(3, corr, it, False)
            diff = fhat - (g - gm) / gn
        corr = float(diff @ diff)
        if optimizer == 0:
            grad = (diff @ sd) * (1.0 if ssd else 2.0 / fn)
            dp = -np.linalg.solve(hess, grad)
        else:
            dgx, dgy = spline_gradients(coef, qk, wx, wy, w, h, degree, BORDER)
            if order == 1:
                a00, a01, a10, a11 = 1 + p[2], p[3], p[4], 1 + p[5]
            else:
                a00 = 1 + p[2] + p[6] * lx + p[7] * ly
                a01 = p[3] + p[7] * lx + p[8] * ly
                a10 = p[4] + p[9] * lx + p[10] * ly
                a11 = 1 + p[5] + p[10] * lx + p[11] * ly
            sd = sd_rows(dgx * a00 + dgy * a10, dgx * a01 + dgy * a11, lx, ly, order)
            hess = sd.T @ sd * (1.0 if ssd else 2.0 / (fn * fn))
            grad = (diff @ sd) * (1.0 if ssd else 2.0 / fn)
            if damping:
                hess = hess + 1e-4 * np.max(np.diag(hess)) * np.eye(npar)
            dp = np.linalg.solve(hess, grad)
        if not np.all(np.isfinite(dp)):
            return out(3, corr, it, False)
        dn = float(np.linalg.norm(dp))
        dn_test = dn
        if optimizer == 1 and dn > cap:
            dp = dp * (cap / dn)
            if test_capped:
                dn_test = cap
        if optimizer == 0:
            p = ic_update(p, dp) if order == 1 else ic_update2(p, dp)
        else:
            p = compose1(p, dp) if order == 1 else compose2(p, dp)
        if not np.all(np.isfinite(p)):
            return out(3, corr, it, False)
        if dn_test < THRESHOLD:
            converged = True
            break
    if not converged and math.isfinite(corr):
        converged = True
    return out(0 if converged else 1, corr, it, converged)


# (name, optimizer 0 icgn / 1 fgn, shape order, ssd)
VARIANTS = [("icgn1_ssd", 0, 1, True), ("icgn2_znssd", 0, 2, False), ("icgn2_ssd", 0, 2, True),
            ("fgn1_ssd", 1, 1, True), ("fgn2_znssd", 1, 2, False), ("fgn2_ssd", 1, 2, True)]
VARIANTS_OUT = os.path.join(HERE, "subset_variants_256.npz")


def bump_pair():
    from traditional_dic_gb300 import synthetic
    f = synthetic.Field("bump", dict(cx=128.0, cy=128.0, s=60.0, a=3.0))
    return synthetic.speckle_pair((256, 256), 1500, f, 0.5, synthetic.BASE_SEED + 17)


def main_variants():
    from traditional_dic_gb300 import synthetic
    qk = qk_matrix(DEGREE)
    pts = [(x, y) for y in range(20, 240, 22) for x in range(20, 240, 22)] + [(5.0, 128.0)]
    arrays = {}
    for tag, pair in (("a", synthetic.workload(0)), ("b", bump_pair())):
        ref, de = pair.reference, pair.deformed
        coef = coefficients(de, DEGREE, BORDER)
        pois = []
        for x, y in pts:
            u, v = pair.field.uv(np.float64(x), np.float64(y))
            pois.append((x, y, round(2 * float(u)) / 2.0, round(2 * float(v)) / 2.0))
        pois = np.array(pois, np.float64)
        arrays[f"reference_{tag}"] = ref
        arrays[f"deformed_{tag}"] = de
        arrays[f"pois_{tag}"] = pois
        for name, opt, order, ssd in VARIANTS:
            res = []
            for x, y, u0, v0 in pois:
                p, corr, iters, status, conv = solve_variant(ref, coef, qk, x, y, (u0, v0), opt, order, ssd)
                res.append(np.concatenate([p, [corr, iters, status, float(conv)]]))
            arrays[f"{name}_{tag}"] = np.array(res, np.float64)
            print(f"{name} {tag}: {int(sum(r[15] for r in res))} converged")
    arrays["settings"] = np.array([DEGREE, BORDER, RADIUS, MAX_ITER, THRESHOLD])
    np.savez_compressed(VARIANTS_OUT, **arrays)
    print(f"wrote {VARIANTS_OUT}")


MASKED_OUT = os.path.join(HERE, "subset_masked_256.npz")
MASKED = [("icgn1_znssd", 0, 1, False), ("icgn2_ssd", 0, 2, True), ("fgn1_ssd", 1, 1, True),
          ("fgn2_znssd", 1, 2, False)]


def disc_roi(h, w):
    yy, xx = np.mgrid[:h, :w]
    return ((xx - 140) ** 2 + (yy - 120) ** 2) < 95 ** 2


def main_masked():
    from traditional_dic_gb300 import synthetic
    qk = qk_matrix(DEGREE)
    pair = synthetic.workload(0)
    ref, de = pair.reference, pair.deformed
    h, w = ref.shape
    roi = disc_roi(h, w)
    coef = coefficients(de, DEGREE, BORDER)
    pts = [(x, y) for y in range(3, 256, 19) for x in range(3, 256, 19)]
    pois = []
    for x, y in pts:
        u, v = pair.field.uv(np.float64(x), np.float64(y))
        pois.append((x, y, round(2 * float(u)) / 2.0, round(2 * float(v)) / 2.0))
    pois = np.array(pois, np.float64)
    arrays = {"roi": roi, "pois": pois, "settings": np.array([DEGREE, BORDER, RADIUS, MAX_ITER, THRESHOLD])}
    for name, opt, order, ssd in MASKED:
        res = []
        for x, y, u0, v0 in pois:
            p, corr, iters, status, conv = solve_variant(ref, coef, qk, x, y, (u0, v0), opt, order, ssd, roi=roi)
            res.append(np.concatenate([p, [corr, iters, status, float(conv)]]))
        arrays[name] = np.array(res, np.float64)
        print(f"masked {name}: {int(sum(r[15] for r in res))} converged of {len(res)}")
    np.savez_compressed(MASKED_OUT, **arrays)
    print(f"wrote {MASKED_OUT}")


PROPAGATION_OUT = os.path.join(HERE, "subset_propagation_256.npz")
SPACING, MAX_ZNSSD = 9, 0.5


def round_half_away(x):
    """std::round / std::llround: halves away from zero."""
    return int(math.copysign(math.floor(abs(x) + 0.5), x))


def propagate_heap(ref, coef, qk, seed_xy, seed_p, seed_corr, roi=None, masked=False, optimizer=0, order=1):
    """ReliabilityPropagation::propagate with one seed and the first-order ZNSSD ICGN (masked by
    ``roi`` when ``masked``: solve_with_mask).  Returns the grid arrays (p: the six first-order
    then the six second-order parameters; correlation, valid, status, iterations; defaults where
    no result was kept), the number of points kept and the number of solves."""
    h, w = ref.shape
    step = SPACING + 1
    gw, gh = -(-w // step), -(-h // step)
    n = gw * gh
    p_out, corr_out = np.zeros((n, 12)), np.zeros(n)
    valid, status, iters = np.zeros(n, bool), np.full(n, -1, np.int64), np.zeros(n, np.int64)
    calc = np.zeros(n, bool)
    roi_ok = (lambda x, y: True) if roi is None else (lambda x, y: bool(roi[y, x]))
    solve = lambda x, y, p0: solve_variant(ref, coef, qk, float(x), float(y), np.asarray(p0, np.float64), optimizer,
                                           order, False, roi=roi if masked else None)
    sxr, syr = round_half_away(seed_xy[0]), round_half_away(seed_xy[1])
    if not (0 <= sxr < w and 0 <= syr < h) or not roi_ok(sxr, syr):
        return p_out, corr_out, valid, status, iters, 0, 0
    gxs = min(max(round_half_away(sxr / step), 0), gw - 1)
    gys = min(max(round_half_away(syr / step), 0), gh - 1)
    sx, sy = gxs * step, gys * step
    if not roi_ok(sx, sy):
        return p_out, corr_out, valid, status, iters, 0, 0
    sidx = gys * gw + gxs
    solves = 0
    sp, scorr, sit = np.concatenate([np.asarray(seed_p, np.float64), np.zeros(6)]), float(seed_corr), 0
    if (sx, sy) != (sxr, syr):
        q, scorr, sit, st, _ = solve(sx, sy, seed_p)
        solves += 1
        sp = q[:12]
        if st != 0 or not (np.all(np.isfinite(sp[:6])) and math.isfinite(scorr)):
            return p_out, corr_out, valid, status, iters, 0, solves
    calc[sidx] = True
    p_out[sidx], corr_out[sidx], valid[sidx], status[sidx], iters[sidx] = sp, scorr, True, 0, sit
    kept = 1
    import heapq
    heap, seq, keys = [(max(0.0, scorr), 0, gxs, gys, sp)], 1, {max(0.0, scorr)}
    while heap:
        _, _, gx, gy, pp = heapq.heappop(heap)
        px, py = gx * step, gy * step
        for nx, ny in ((px, py - step), (px + step, py), (px, py + step), (px - step, py)):
            if not (0 <= nx < w and 0 <= ny < h):
                continue
            gnx, gny = nx // step, ny // step
            if gnx >= gw or gny >= gh:
                continue
            nidx = gny * gw + gnx
            if calc[nidx]:
                continue
            if not roi_ok(nx, ny) or nx - RADIUS < 0 or ny - RADIUS < 0 or nx + RADIUS >= w or ny + RADIUS >= h:
                calc[nidx] = True
                continue
            dx, dy = float(nx - px), float(ny - py)
            p0 = np.array([pp[0] + pp[2] * dx + pp[3] * dy, pp[1] + pp[4] * dx + pp[5] * dy,
                           pp[2], pp[3], pp[4], pp[5]])
            q, c, it, st, _ = solve(nx, ny, p0)
            solves += 1
            calc[nidx] = True
            r = q[:6]
            if (st == 0 and c < MAX_ZNSSD and abs(p0[0] - r[0]) < step and abs(p0[1] - r[1]) < step
                    and np.all(np.isfinite(r)) and math.isfinite(c)):
                p_out[nidx], corr_out[nidx], valid[nidx], status[nidx], iters[nidx] = q[:12], c, True, st, it
                kept += 1
                # the heap order of equal keys is implementation-defined in std::priority_queue
                assert c not in keys, "two equal ZNSSD keys: the visit order would be ambiguous"
                keys.add(c)
                heapq.heappush(heap, (c, seq, gnx, gny, r))
                seq += 1
    return p_out, corr_out, valid, status, iters, kept, solves


def main_propagation():
    from traditional_dic_gb300 import synthetic
    qk = qk_matrix(DEGREE)
    pair = synthetic.workload(0)
    ref, de = pair.reference, pair.deformed
    coef = coefficients(de, DEGREE, BORDER)
    seed_xy = (131.4, 126.0)   # rounds to (131, 126), off the grid: the seed is solved again at (130, 130)
    u, v = pair.field.uv(np.float64(seed_xy[0]), np.float64(seed_xy[1]))
    seed_p = np.array([round(2 * float(u)) / 2.0, round(2 * float(v)) / 2.0, 0, 0, 0, 0])
    yy, xx = np.mgrid[:256, :256]
    rois = {"full": None, "roi": ((xx - 120) ** 2 + (yy - 140) ** 2 < 90 ** 2) & ~((xx > 60) & (xx < 75))}
    arrays = {"seed_xy": np.array(seed_xy), "seed_p": seed_p, "seed_correlation": np.array(0.0),
              "settings": np.array([DEGREE, BORDER, RADIUS, MAX_ITER, THRESHOLD, SPACING, MAX_ZNSSD])}
    # the full grid again with the FGN solver and with the second-order ICGN (ZNSSD both): the
    # guesses carry the six first-order parameters, the second-order terms start at zero
    runs = [(tag, roi, 0, 1) for tag, roi in rois.items()] + [("fgn", None, 1, 1), ("icgn2", None, 0, 2)]
    for tag, roi, opt, order in runs:
        p, c, val, st, it, kept, solves = propagate_heap(ref, coef, qk, seed_xy, seed_p, 0.0, roi, optimizer=opt,
                                                         order=order)
        arrays[f"p_{tag}"], arrays[f"correlation_{tag}"], arrays[f"valid_{tag}"] = p, c, val
        arrays[f"status_{tag}"], arrays[f"iterations_{tag}"] = st, it
        arrays[f"counts_{tag}"] = np.array([kept, solves])
        if roi is not None:
            arrays[f"mask_{tag}"] = roi
        print(f"propagation {tag}: {kept} kept of {solves} solves")
    np.savez_compressed(PROPAGATION_OUT, **arrays)
    print(f"wrote {PROPAGATION_OUT}")


SEED_OUT = os.path.join(HERE, "subset_seed_256.npz")
# integer search: subset radius, search radius, pyramid scale, pyramid refinement radius;
# seed selection: seed count, k-means iterations, sample limit, max ZNSSD, min texture std,
# min displacement norm.  The subpixel ICGN uses RADIUS, MAX_ITER and THRESHOLD.
IS_RADIUS, IS_SEARCH, PYR_SCALE, PYR_REFINE = 10, 20, 4, 4
SEED_COUNT, KMEANS_ITERS, SAMPLE_LIMIT, SEED_MAX_ZNSSD, MIN_TEXTURE, MIN_NORM = 64, 20, 20000, 0.3, 0.02, 0.0
MIN_VALID_SAMPLES, MIN_VALID_RATIO = 12, 0.5   # SubsetConfig defaults; the masked ICGN above uses the same
TIE = 1e-12


def llround_pos(x):
    return int(math.floor(x + 0.5))


def texture_std(ref, x, y):
    r = IS_RADIUS
    h, w = ref.shape
    if x - r < 0 or y - r < 0 or x + r >= w or y + r >= h:
        return 0.0
    win = ref[y - r:y + r + 1, x - r:x + r + 1].astype(np.float64)
    n = win.size
    mean = win.sum() / n
    return math.sqrt(max(0.0, (win * win).sum() / n - mean * mean))


def seed_candidates(ref, roi, truncate=False):
    h, w = ref.shape
    # max(integer-search radius, subpixel radius), plus the search radius with truncated subsets
    margin = IS_RADIUS + (IS_SEARCH if truncate else 0)
    full = len(circle(IS_RADIUS))

    def ok(x, y):   # is_candidate_margin_valid (seed_selector.cpp:440-476)
        if not (margin <= x < w - margin and margin <= y < h - margin):
            return False
        if not truncate:
            return True
        c = circle(IS_RADIUS)
        kept = int(roi[y + c[:, 1], x + c[:, 0]].sum())
        return kept >= max(6, max(MIN_VALID_SAMPLES, math.ceil(MIN_VALID_RATIO * full)))

    ys, xs = np.nonzero(roi)                      # row-major: y outer, x inner
    keep = (xs >= margin) & (xs < w - margin) & (ys >= margin) & (ys < h - margin)
    pts = np.column_stack([xs[keep], ys[keep]])
    assert len(pts), "no candidate point"
    if len(pts) > SAMPLE_LIMIT:
        step = (len(pts) - 1) / (SAMPLE_LIMIT - 1)
        pts = pts[[min(llround_pos(i * step), len(pts) - 1) for i in range(SAMPLE_LIMIT)]]
    count = min(SEED_COUNT, len(pts))
    step = 0.0 if count == 1 else (len(pts) - 1) / (count - 1)
    centres = pts[[min(llround_pos(i * step), len(pts) - 1) for i in range(count)]].astype(np.float64)
    px, py = pts[:, 0].astype(np.float64), pts[:, 1].astype(np.float64)
    for _ in range(KMEANS_ITERS):
        d2 = (px[:, None] - centres[None, :, 0]) ** 2 + (py[:, None] - centres[None, :, 1]) ** 2
        best = np.argmin(d2, axis=1)               # the first centre on ties
        for i in range(count):
            sel = best == i
            if sel.any():
                centres[i] = [px[sel].sum() / sel.sum(), py[sel].sum() / sel.sum()]   # integer sums: exact
    cands = []
    for cx, cy in centres:
        rx, ry = llround_pos(cx), llround_pos(cy)
        if 0 <= rx < w and 0 <= ry < h and roi[ry, rx] and ok(rx, ry) and texture_std(ref, rx, ry) >= MIN_TEXTURE:
            cands.append((rx, ry))
            continue
        d = (px - cx) ** 2 + (py - cy) ** 2
        order = np.argsort(d, kind="stable")
        lim = min(50, len(order))
        assert lim == len(order) or d[order[lim - 1]] != d[order[lim]], "distance tie at the 50-point cut"
        tex = [texture_std(ref, int(pts[j, 0]), int(pts[j, 1])) for j in order[:lim]]
        k = int(np.argmax(tex))
        assert sum(t == tex[k] for t in tex) == 1, "texture tie among the nearest points"
        cands.append((int(pts[order[k], 0]), int(pts[order[k], 1])))
    return np.array(cands, np.int64)


def circle(r, step=1):
    return np.array([(dx, dy) for dy in range(-r, r + 1, step) for dx in range(-r, r + 1, step)
                     if dx * dx + dy * dy <= r * r], np.int64)


def scan(de, cx, cy, offs, fvals, us, vs):
    """Best (u, v, zncc) over the displacements us x vs in scan order (v outer, u inner), with the
    second best ZNCC; positions whose subset leaves the image are skipped."""
    h, w = de.shape
    r = IS_RADIUS
    uu, vv = np.meshgrid(us, vs)
    uu, vv = uu.ravel(), vv.ravel()
    inb = (cx + uu - r >= 0) & (cy + vv - r >= 0) & (cx + uu + r < w) & (cy + vv + r < h)
    uu, vv = uu[inb], vv[inb]
    if uu.size == 0:
        return None
    fm = fvals.sum() / len(fvals)
    fd = fvals - fm
    fn = (fd * fd).sum()
    if fn <= EPS:
        return None
    g = de[cy + vv[:, None] + offs[None, :, 1], cx + uu[:, None] + offs[None, :, 0]].astype(np.float64)
    gd = g - (g.sum(axis=1) / g.shape[1])[:, None]
    dn = (gd * gd).sum(axis=1)
    z = np.where(dn <= EPS, -np.inf, (gd @ fd) / np.sqrt(fn * np.maximum(dn, EPS)))
    k = int(np.argmax(z))
    if not np.isfinite(z[k]):
        return None
    rest = np.delete(z, k)
    second = rest.max() if rest.size else -np.inf
    assert z[k] - second > TIE, "two integer displacements within 1e-12 ZNCC"
    return int(uu[k]), int(vv[k]), float(z[k])


def integer_search(ref, de, x, y, roi=None):
    """estimate_with_interpolators, or estimate_with_mask_interpolators when ``roi`` is given:
    samples outside the image or the ROI dropped, at least max(12, ceil(half the circle)) kept."""
    h, w = ref.shape
    r = IS_RADIUS
    full, coarse = circle(r), circle(r, PYR_SCALE)
    if roi is None:
        if x - r < 0 or y - r < 0 or x + r >= w or y + r >= h:
            return None
    else:
        if not roi[y, x]:
            return None
        need = lambda c: max(12, math.ceil(0.5 * len(c)))
        keep = lambda c: c[(x + c[:, 0] >= 0) & (x + c[:, 0] < w) & (y + c[:, 1] >= 0) & (y + c[:, 1] < h)]
        full_all, coarse_all = full, coarse
        full, coarse = keep(full), keep(coarse)
        full = full[roi[y + full[:, 1], x + full[:, 0]]]
        coarse = coarse[roi[y + coarse[:, 1], x + coarse[:, 0]]]
        if len(full) < need(full_all):
            return None
    f = ref[y + full[:, 1], x + full[:, 0]].astype(np.float64)
    fc = ref[y + coarse[:, 1], x + coarse[:, 0]].astype(np.float64)
    min_u, max_u, min_v, max_v = r - x, w - 1 - r - x, r - y, h - 1 - r - y
    best = None
    coarse_ok = roi is None or len(coarse) >= need(coarse_all)
    if roi is not None:
        fd = f - f.sum() / len(f)
        if (fd * fd).sum() <= EPS:
            return None
    if min_u <= max_u and min_v <= max_v and coarse_ok:
        c = scan(de, x, y, coarse, fc, np.arange(min_u, max_u + 1, PYR_SCALE), np.arange(min_v, max_v + 1, PYR_SCALE))
        if c is not None:
            rr = max(max(PYR_REFINE, math.ceil(1.5 * r)), PYR_SCALE)
            best = scan(de, x, y, full, f, np.arange(max(min_u, c[0] - rr), min(max_u, c[0] + rr) + 1),
                        np.arange(max(min_v, c[1] - rr), min(max_v, c[1] + rr) + 1))
    if IS_SEARCH > 0:
        local = scan(de, x, y, full, f, np.arange(-IS_SEARCH, IS_SEARCH + 1), np.arange(-IS_SEARCH, IS_SEARCH + 1))
        if local is not None:
            if best is not None:
                assert abs(local[2] + 0.02 - best[2]) > TIE, "local preference decided by a near tie"
            if best is None or local[2] + 0.02 >= best[2]:
                best = local
    return best


def select_seed(ref, de, roi, truncate=False):
    qk = qk_matrix(DEGREE)
    h, w = ref.shape
    ys, xs = np.arange(-BORDER, h + BORDER), np.arange(-BORDER, w + BORDER)
    lazy = de[np.ix_(np.clip(ys, 0, h - 1), np.clip(xs, 0, w - 1))].astype(np.float64)   # clamp padding, no deconvolution
    cands = seed_candidates(ref, roi, truncate)
    integer = np.full((len(cands), 4), np.nan)      # u, v, zncc, found
    evals = np.full((len(cands), 9), np.nan)        # p[6], quality, refined, valid
    best = -1
    for i, (x, y) in enumerate(cands):
        it = integer_search(ref, de, int(x), int(y), roi if truncate else None)
        integer[i] = (np.nan, np.nan, np.nan, 0) if it is None else (it[0], it[1], it[2], 1)
        if it is None:
            evals[i, 7:] = (0, 0)
            continue
        q, corr, _, st, _ = solve_variant(ref, lazy, qk, float(x), float(y), (float(it[0]), float(it[1])), 0, 1, False,
                                          roi=roi if truncate else None)
        if st == 0 and np.all(np.isfinite(q[:6])) and math.isfinite(corr):
            evals[i, :6], evals[i, 6], evals[i, 7] = q[:6], corr, 1
        else:
            zn = max(0.0, 2.0 * (1.0 - max(-1.0, min(1.0, it[2]))))
            evals[i, :6], evals[i, 6], evals[i, 7] = (it[0], it[1], 0, 0, 0, 0), zn, 0
        evals[i, 8] = 1
        quality, norm = evals[i, 6], math.hypot(evals[i, 0], evals[i, 1])
        if quality <= SEED_MAX_ZNSSD and norm >= MIN_NORM:
            if best < 0:
                best = i
                continue
            cur = evals[best, 6]
            assert abs(abs(quality - cur) - 1e-9) > TIE, "seed ranking decided by a near tie"
            if quality < cur - 1e-9 or (quality <= cur + 1e-9 and norm > math.hypot(evals[best, 0], evals[best, 1])):
                best = i
    return cands, integer, evals, best


def main_seed():
    from traditional_dic_gb300 import synthetic
    assert (RADIUS, MAX_ITER, THRESHOLD) == (IS_RADIUS, 20, 1e-3)   # the subpixel ICGN settings
    pair = synthetic.workload(0)
    ref, de = pair.reference, pair.deformed
    yy, xx = np.mgrid[:256, :256]
    rois = {"full": np.ones((256, 256), bool), "roi": (xx - 150) ** 2 + (yy - 110) ** 2 < 70 ** 2,
            # truncated subsets: masked integer search and refinement, margin radius + search radius
            "truncated": ((xx - 128) ** 2 + (yy - 128) ** 2 < 95 ** 2) & ~((xx > 100) & (xx < 108))}
    arrays = {"settings": np.array([IS_RADIUS, IS_SEARCH, PYR_SCALE, PYR_REFINE, SEED_COUNT, KMEANS_ITERS,
                                    SAMPLE_LIMIT, SEED_MAX_ZNSSD, MIN_TEXTURE, MIN_NORM, DEGREE, BORDER, RADIUS,
                                    MAX_ITER, THRESHOLD])}
    for tag, roi in rois.items():
        cands, integer, evals, best = select_seed(ref, de, roi, truncate=tag == "truncated")
        arrays[f"candidates_{tag}"], arrays[f"integer_{tag}"], arrays[f"evaluations_{tag}"] = cands, integer, evals
        arrays[f"best_{tag}"] = np.array(best)
        if tag != "full":
            arrays[f"mask_{tag}"] = roi
        print(f"seed {tag}: {len(cands)} candidates, {int(np.nansum(evals[:, 7]))} refined, best {best} at "
              f"{tuple(cands[best]) if best >= 0 else None}")
    np.savez_compressed(SEED_OUT, **arrays)
    print(f"wrote {SEED_OUT}")


TRUNCATED_OUT = os.path.join(HERE, "subset_truncated_256.npz")


def mirror_index(i, n):
    """padding.cpp:11-24."""
    if n <= 1:
        return 0
    while i < 0 or i >= n:
        i = -i - 1 if i < 0 else 2 * n - i - 1
    return i


def subset_compute_truncated(ref, de, roi):
    """SubsetDIC::compute with truncate_roi_subsets (subset_dic.cpp:39-105): images mirror-padded
    and the ROI zero-padded by recommended_subset_padding (padding.cpp:28-36), the seed selected and
    the grid propagated on the padded images with masked subsets, then the grid points inside the
    original image returned, shifted back by the padding."""
    h, w = ref.shape
    pad = IS_SEARCH + max(RADIUS, IS_RADIUS, RADIUS) + BORDER
    ys = [mirror_index(y - pad, h) for y in range(h + 2 * pad)]
    xs = [mirror_index(x - pad, w) for x in range(w + 2 * pad)]
    pref, pdef = ref[np.ix_(ys, xs)], de[np.ix_(ys, xs)]
    proi = np.zeros((h + 2 * pad, w + 2 * pad), bool)
    proi[pad:pad + h, pad:pad + w] = roi
    cands, _, evals, best = select_seed(pref, pdef, proi, truncate=True)
    assert best >= 0, "no seed"
    seed_xy, seed_p, seed_corr = cands[best].astype(np.float64), evals[best, :6], evals[best, 6]
    coef = coefficients(pdef, DEGREE, BORDER)
    p, c, val, st, it, kept, solves = propagate_heap(pref, coef, qk_matrix(DEGREE), seed_xy, seed_p, seed_corr,
                                                      roi=proi, masked=True)
    assert kept > 0
    step = SPACING + 1
    gw = -(-(w + 2 * pad) // step)
    n = len(val)
    gx, gy = (np.arange(n) % gw) * step - pad, (np.arange(n) // gw) * step - pad
    inside = (gx >= 0) & (gy >= 0) & (gx < w) & (gy < h)
    return dict(x=gx[inside].astype(np.float64), y=gy[inside].astype(np.float64), p=p[inside], correlation=c[inside],
                valid=val[inside], iterations=it[inside], seed=np.concatenate([seed_xy, seed_p, [seed_corr]]),
                counts=np.array([kept, solves, pad]))


def main_truncated():
    from traditional_dic_gb300 import synthetic
    pair = synthetic.workload(0)
    ref, de = pair.reference, pair.deformed
    yy, xx = np.mgrid[:256, :256]
    rois = {"full": np.ones((256, 256), bool),
            "roi": ((xx - 140) ** 2 + (yy - 120) ** 2 < 110 ** 2) & ~((xx > 40) & (xx < 52) & (yy > 100))}
    arrays = {}
    for tag, roi in rois.items():
        out = subset_compute_truncated(ref, de, roi)
        for k, v in out.items():
            arrays[f"{k}_{tag}"] = v
        if tag != "full":
            arrays[f"mask_{tag}"] = roi
        edge = (out["x"] < RADIUS) | (out["y"] < RADIUS) | (out["x"] >= 256 - RADIUS) | (out["y"] >= 256 - RADIUS)
        print(f"truncated {tag}: {len(out['x'])} points, {int(out['valid'].sum())} valid, "
              f"{int(out['valid'][edge].sum())} valid within a radius of the image edge; kept/solves/pad {out['counts']}")
    np.savez_compressed(TRUNCATED_OUT, **arrays)
    print(f"wrote {TRUNCATED_OUT}")


DEGREE5_OUT = os.path.join(HERE, "subset_degree5_256.npz")
DEGREE5 = [("icgn1_znssd", 0, 1, False), ("fgn1_znssd", 1, 1, False), ("icgn2_znssd", 0, 2, False),
           ("fgn2_ssd", 1, 2, True)]


def main_degree5():
    """The quintic B-spline (degree 5, the reference's default): coefficients and four routes on
    the small workload's POIs."""
    from traditional_dic_gb300 import synthetic
    qk = qk_matrix(5)
    pair = synthetic.workload(0)
    ref, de = pair.reference, pair.deformed
    coef = coefficients(de, 5, BORDER)
    pts = [(x, y) for y in range(20, 240, 22) for x in range(20, 240, 22)] + [(5.0, 128.0)]
    pois = []
    for x, y in pts:
        u, v = pair.field.uv(np.float64(x), np.float64(y))
        pois.append((x, y, round(2 * float(u)) / 2.0, round(2 * float(v)) / 2.0))
    pois = np.array(pois, np.float64)
    arrays = {"pois": pois, "coef_crop": coef[:40, :40], "settings": np.array([5, BORDER, RADIUS, MAX_ITER, THRESHOLD])}
    for name, opt, order, ssd in DEGREE5:
        res = []
        for x, y, u0, v0 in pois:
            p, corr, iters, status, conv = solve_variant(ref, coef, qk, x, y, (u0, v0), opt, order, ssd, degree=5)
            res.append(np.concatenate([p, [corr, iters, status, float(conv)]]))
        arrays[name] = np.array(res, np.float64)
        print(f"degree 5 {name}: {int(sum(r[15] for r in res))} converged")
    np.savez_compressed(DEGREE5_OUT, **arrays)
    print(f"wrote {DEGREE5_OUT}")


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
    main_variants()
    main_masked()
    main_propagation()
    main_seed()
    main_truncated()
    main_degree5()


if __name__ == "__main__":
    main()
