"""The arguments the seed search's kernels rest on, checked on the CPU.

* Coarse lattice: with circle offsets (dx, dy) that start at -r in steps of cstep
  (circle_offsets) and positions u = r - cx + cstep * ui (min_u = r - cx), every deformed sample
  x = cx + u + dx is a multiple of cstep inside [0, w), and its lattice index
  x / cstep = ui + (dx + r) / cstep lies inside the decimated image ((w - 1) / cstep + 1 wide);
  likewise in y.  The coarse kernel reads the decimated copy at exactly these indices.
* k-means filter: for centres rounded to float and distances rounded in float (no fused
  multiply-add), |d32 - d64| stays below err32 = 1e-6 (C (|dx32| + |dy32|) + d32) + 16 (2^-24 C)^2
  + 1e-6, C above every coordinate, up to C = 2^22; err32 is what the kernel allows, so the FP64
  minimum is always among the centres it rescores.
* One-pass coarse search: rescoring near each tile's FP32 maximum picks the winner that
  rescoring near the candidate's FP32 maximum picks."""
import numpy as np
import pytest


def _circle_offsets(r, step):
    return [(dx, dy) for dy in range(-r, r + 1, step) for dx in range(-r, r + 1, step) if dx * dx + dy * dy <= r * r]


@pytest.mark.parametrize("r,cstep,w,h", [(10, 4, 2048, 2048), (7, 3, 200, 180), (15, 5, 333, 97), (10, 1, 64, 64),
                                          (20, 4, 5120, 301), (9, 2, 41, 40)])
def test_coarse_samples_lie_on_the_decimated_lattice(r, cstep, w, h):
    rng = np.random.default_rng(r * 100 + cstep)
    offs = _circle_offsets(r, cstep)
    dw, dh = (w - 1) // cstep + 1, (h - 1) // cstep + 1
    for _ in range(40):
        cx, cy = int(rng.integers(r, w - r)), int(rng.integers(r, h - r))
        min_u, max_u, min_v, max_v = r - cx, w - 1 - r - cx, r - cy, h - 1 - r - cy
        nu, nv = (max_u - min_u) // cstep + 1, (max_v - min_v) // cstep + 1
        for ui in (0, nu // 2, nu - 1):
            for vi in (0, nv // 3, nv - 1):
                u, v = min_u + cstep * ui, min_v + cstep * vi
                for dx, dy in offs:
                    x, y = cx + u + dx, cy + v + dy
                    assert 0 <= x < w and 0 <= y < h
                    assert x % cstep == 0 and y % cstep == 0
                    a, b = (dx + r) // cstep, (dy + r) // cstep
                    assert (dx + r) % cstep == 0 and (dy + r) % cstep == 0
                    assert ui + a == x // cstep < dw and vi + b == y // cstep < dh


@pytest.mark.parametrize("big", [100, 2048, 5120, 8192, 1 << 16, (1 << 22) - 1])
def test_kmeans_fp32_error_bound(big):
    rng = np.random.default_rng(big)
    n = 200_000
    px, py = rng.integers(0, big + 1, n), rng.integers(0, big + 1, n)
    cx, cy = rng.uniform(0, big, n), rng.uniform(0, big, n)
    near = rng.random(n) < 0.5                       # centres next to their points: tiny distances
    cx[near] = np.clip(px[near] + rng.normal(0, 1e-3, near.sum()), 0, big)
    cy[near] = np.clip(py[near] + rng.normal(0, 1e-3, near.sum()), 0, big)
    f = np.float32
    cb = f(big + 1)
    ucb = np.ldexp(float(big + 1), -24)
    kabs = f(16.0 * ucb * ucb + 1e-6)
    dx = (px.astype(f) - cx.astype(f)).astype(f)
    dy = (py.astype(f) - cy.astype(f)).astype(f)
    d32 = ((dx * dx).astype(f) + (dy * dy).astype(f)).astype(f)
    err = (f(1e-6) * (cb * (np.abs(dx) + np.abs(dy)) + d32) + kabs).astype(f)
    ddx, ddy = px - cx, py - cy
    d64 = ddx * ddx + ddy * ddy
    assert np.all(np.abs(d32.astype(np.float64) - d64) <= 0.25 * err.astype(np.float64))   # four times over


def _argmax_first(z, idx):
    """The winner of the search's rule: the largest FP64 score, the first in scan order on ties."""
    if len(idx) == 0:
        return None
    best = max(z[i] for i in idx)
    return min(i for i in idx if z[i] == best)


@pytest.mark.parametrize("seed", range(12))
def test_one_pass_tile_threshold_picks_the_two_pass_winner(seed):
    """The coarse search's one pass rescores, per tile, the positions within the margin of the
    tile's FP32 maximum; the two-pass search rescores the positions within the margin of the
    candidate's FP32 maximum.  With FP32 scores within margin / 2 of the FP64 ones, both pick the
    same position (ties to the first in scan order), on score surfaces with plateaus and ties."""
    rng = np.random.default_rng(seed)
    margin, err = 1e-3, 4e-5
    npos, per_tile = int(rng.integers(500, 20000)), int(rng.choice([64, 256, 4096]))
    z64 = rng.uniform(-0.3, 0.6, npos)
    peak = rng.integers(0, npos, 3)
    z64[peak] = 0.95                                              # tied maxima
    near = rng.integers(0, npos, 40)
    z64[near] = 0.95 - rng.uniform(0, 2 * margin, 40)             # close runners-up
    z64 = np.round(z64, int(rng.choice([3, 6, 12])))              # plateaus: many equal scores
    z32 = z64 + rng.uniform(-err, err, npos)
    two_pass = [i for i in range(npos) if z32[i] >= z32.max() - margin]
    one_pass = []
    for t0 in range(0, npos, per_tile):
        tile = range(t0, min(npos, t0 + per_tile))
        tmax = max(z32[i] for i in tile)
        one_pass += [i for i in tile if z32[i] >= tmax - margin]
    assert set(two_pass) <= set(one_pass)
    assert _argmax_first(z64, one_pass) == _argmax_first(z64, two_pass) == _argmax_first(z64, range(npos))
