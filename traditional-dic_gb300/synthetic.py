"""Seeded synthetic speckle pairs for the five benchmark workloads.

No public dataset is involved.  A reference image is
``I(x, y) = 30 + sum_k A_k exp(-((x - x_k)^2 + (y - y_k)^2) / (2 sigma_k^2))`` clipped to the
dtype range (8-bit: [0, 255]; 16-bit: amplitudes and background x256, [0, 65535]).  The deformed
image is the same analytic function sampled at the inverse-mapped coordinates X solving
``X + u(X) = x`` (five fixed-point iterations), plus N(0, sigma_n) gray-level noise, rounded and
clipped.  Ground-truth displacements and their gradients are analytic.

Workloads (numpy ``default_rng(20261203 + index)``):
  0: 256^2 uint8, 1500 blobs, sigma U[2,4], u = 2.3 + 0.001 x, v = -1.7 - 0.0005 y, noise 0.5
  1: 2048^2 uint8, 24000 blobs, u = 0.5 sin(2 pi x / 256), v = 0.3 cos(2 pi y / 192), noise 1
  2: side log-U[512, 4096], affine (translation U(-5, 5), gradients U(-0.01, 0.01)), noise 1
  4: 5120^2 uint16, 150000 blobs, sigma U[1.5, 5], u = 0.02 (y - c) + 4 g(x, y) + 0.2 sin(2 pi x / 64),
     v = 2 g(x, y) with g a Gaussian bump of sigma 600 at the centre, noise 2
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BASE_SEED = 20261203


@dataclass
class Field:
    """Analytic displacement u(X, Y), v(X, Y) in reference coordinates with gradients."""
    kind: str
    params: dict = field(default_factory=dict)

    def uv(self, X, Y):
        p = self.params
        if self.kind == "linear":
            return p["u0"] + p["ux"] * X + p["uy"] * Y, p["v0"] + p["vx"] * X + p["vy"] * Y
        if self.kind == "sine":
            return (p["au"] * np.sin(2 * np.pi * X / p["lu"]) + 0.0 * Y,
                    p["av"] * np.cos(2 * np.pi * Y / p["lv"]) + 0.0 * X)
        if self.kind == "bump":
            g = np.exp(-((X - p["cx"]) ** 2 + (Y - p["cy"]) ** 2) / (2 * p["s"] ** 2))
            u = p.get("shear", 0.0) * (Y - p["cy"]) + p["a"] * g + p.get("sa", 0.0) * np.sin(2 * np.pi * X / p.get("sl", 64.0))
            return u, 0.5 * p["a"] * g
        raise ValueError(self.kind)

    def gradients(self, X, Y):
        p = self.params
        X = np.asarray(X, np.float64)
        Y = np.asarray(Y, np.float64)
        z = np.zeros_like(X + Y)
        if self.kind == "linear":
            return z + p["ux"], z + p["uy"], z + p["vx"], z + p["vy"]
        if self.kind == "sine":
            return (p["au"] * 2 * np.pi / p["lu"] * np.cos(2 * np.pi * X / p["lu"]) + z, z,
                    z, -p["av"] * 2 * np.pi / p["lv"] * np.sin(2 * np.pi * Y / p["lv"]) + z)
        if self.kind == "bump":
            g = np.exp(-((X - p["cx"]) ** 2 + (Y - p["cy"]) ** 2) / (2 * p["s"] ** 2))
            gx = -g * (X - p["cx"]) / p["s"] ** 2
            gy = -g * (Y - p["cy"]) / p["s"] ** 2
            sl = p.get("sl", 64.0)
            ux = p["a"] * gx + p.get("sa", 0.0) * 2 * np.pi / sl * np.cos(2 * np.pi * X / sl)
            uy = p.get("shear", 0.0) + p["a"] * gy
            return ux + z, uy + z, 0.5 * p["a"] * gx + z, 0.5 * p["a"] * gy + z
        raise ValueError(self.kind)

    def max_grad(self, shape):
        h, w = shape
        ys, xs = np.mgrid[0:h:max(1, h // 64), 0:w:max(1, w // 64)].astype(np.float64)
        return float(max(np.abs(g).max() for g in self.gradients(xs, ys)))


@dataclass
class Pair:
    reference: np.ndarray
    deformed: np.ndarray
    field: Field
    seed: int
    meta: dict

    def truth(self, x, y):
        """Ground truth (u, v, du_dx, du_dy, dv_dx, dv_dy) at reference points."""
        x = np.asarray(x, np.float64)
        y = np.asarray(y, np.float64)
        u, v = self.field.uv(x, y)
        ux, uy, vx, vy = self.field.gradients(x, y)
        return u, v, ux, uy, vx, vy


def _render(shape, cx, cy, sig, amp, Xmap=None, Ymap=None, wcx=None, wcy=None, pad=0, chunk=4096):
    """Sum of Gaussian blobs on the pixel grid; (Xmap, Ymap) give the evaluation coordinates."""
    h, w = shape
    out = np.zeros(h * w, np.float64)
    if wcx is None:
        wcx, wcy = cx, cy
    half = int(math.ceil(5.0 * float(sig.max()))) + pad
    off = np.arange(-half, half + 1)
    K = off.size
    for s in range(0, cx.size, chunk):
        e = min(cx.size, s + chunk)
        bx = np.rint(wcx[s:e]).astype(np.int64)
        by = np.rint(wcy[s:e]).astype(np.int64)
        xs = bx[:, None] + off[None, :]                       # (n, K)
        ys = by[:, None] + off[None, :]
        okx = (xs >= 0) & (xs < w)
        oky = (ys >= 0) & (ys < h)
        xs_c = np.clip(xs, 0, w - 1)
        ys_c = np.clip(ys, 0, h - 1)
        idx = ys_c[:, :, None] * w + xs_c[:, None, :]       # (n, K, K)
        ok = oky[:, :, None] & okx[:, None, :]
        if Xmap is None:
            X = xs_c[:, None, :].astype(np.float64)
            Y = ys_c[:, :, None].astype(np.float64)
        else:
            X = Xmap.ravel()[idx]
            Y = Ymap.ravel()[idx]
        d2 = (X - cx[s:e, None, None]) ** 2 + (Y - cy[s:e, None, None]) ** 2
        val = amp[s:e, None, None] * np.exp(-d2 / (2.0 * sig[s:e, None, None] ** 2))
        val = np.where(ok, val, 0.0)
        out += np.bincount(idx.ravel(), weights=val.ravel(), minlength=h * w)
        del idx, X, Y, d2, val
    return out.reshape(h, w)


def speckle_pair(shape, n_blobs, fld: Field, noise: float, seed: int, dtype=np.uint8,
                 sigma=(2.0, 4.0), amplitude=(40.0, 120.0)) -> Pair:
    rng = np.random.default_rng(seed)
    h, w = shape
    cx = rng.uniform(0, w, n_blobs)
    cy = rng.uniform(0, h, n_blobs)
    sig = rng.uniform(sigma[0], sigma[1], n_blobs)
    amp = rng.uniform(amplitude[0], amplitude[1], n_blobs)
    scale, top = (1.0, 255.0) if dtype == np.uint8 else (256.0, 65535.0)
    ref = 30.0 + _render(shape, cx, cy, sig, amp)
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    X, Y = xs.copy(), ys.copy()
    for _ in range(5):
        u, v = fld.uv(X, Y)
        X = xs - u
        Y = ys - v
    ub, vb = fld.uv(cx, cy)
    pad = int(math.ceil(fld.max_grad(shape) * 5.0 * sigma[1])) + 2
    de = 30.0 + _render(shape, cx, cy, sig, amp, Xmap=X, Ymap=Y, wcx=cx + ub, wcy=cy + vb, pad=pad)
    de = de + rng.normal(0.0, noise, size=de.shape)
    ref_q = np.clip(np.rint(ref * scale), 0, top).astype(dtype)
    de_q = np.clip(np.rint(de * scale), 0, top).astype(dtype)
    return Pair(ref_q, de_q, fld, seed, {"n_blobs": n_blobs, "noise": noise, "dtype": np.dtype(dtype).name})


def workload(index: int, side: int | None = None) -> Pair:
    """The seeded pair of workload ``index`` (0: 256^2, 1: 2048^2, 4: 5120^2).  For workload 1,
    ``side`` renders the same field and speckle density on a side x side image (the blob count
    scales with the area), a smaller case of the same work for profiling."""
    seed = BASE_SEED + index
    if index == 0:
        f = Field("linear", dict(u0=2.3, ux=0.001, uy=0.0, v0=-1.7, vx=0.0, vy=-0.0005))
        return speckle_pair((256, 256), 1500, f, 0.5, seed)
    if index == 1:
        side = side or 2048
        f = Field("sine", dict(au=0.5, lu=256.0, av=0.3, lv=192.0))
        return speckle_pair((side, side), int(round(24000 * (side / 2048.0) ** 2)), f, 1.0, seed)
    if index == 4:
        f = Field("bump", dict(cx=2560.0, cy=2560.0, s=600.0, a=4.0, shear=0.02, sa=0.2, sl=64.0))
        return speckle_pair((5120, 5120), 150000, f, 2.0, seed, dtype=np.uint16, sigma=(1.5, 5.0))
    raise ValueError("use batch_workload() for the uneven batch")


def _batch_pair(args):
    side, dtype_name, params, seed = args
    return speckle_pair((side, side), int(round(24000 * (side / 2048.0) ** 2)), Field("linear", params), 1.0, seed,
                        dtype=np.dtype(dtype_name).type)


def batch_workload(n_pairs: int = 48, seed: int = BASE_SEED + 2, max_side: int = 4096, pool=None):
    """Uneven batch: sides log-U[512, max_side], half uint8 / half uint16, affine fields,
    per-pair radius in {7, 11, 15, 21, 25} and POI step in {3, 5, 8}.  All parameters are drawn
    first from one generator; the pairs (each from its own seed) render in ``pool`` (an
    executor whose workers can import this package) when one is given."""
    rng = np.random.default_rng(seed)
    specs, extra = [], []
    for i in range(n_pairs):
        side = int(round(math.exp(rng.uniform(math.log(512), math.log(max_side)))))
        dtype = np.uint8 if i % 2 == 0 else np.uint16
        params = dict(u0=rng.uniform(-5, 5), ux=rng.uniform(-0.01, 0.01), uy=rng.uniform(-0.01, 0.01),
                      v0=rng.uniform(-5, 5), vx=rng.uniform(-0.01, 0.01), vy=rng.uniform(-0.01, 0.01))
        # centre the affine field so the translation stays within U(-5, 5) over the image
        params["u0"] -= params["ux"] * side / 2 + params["uy"] * side / 2
        params["v0"] -= params["vx"] * side / 2 + params["vy"] * side / 2
        radius = int(rng.choice([7, 11, 15, 21, 25]))
        step = int(rng.choice([3, 5, 8]))
        specs.append((side, np.dtype(dtype).name, params, seed * 1000 + i))
        extra.append((radius, step))
    pairs = list(pool.map(_batch_pair, specs)) if pool is not None else [_batch_pair(a) for a in specs]
    for p, (radius, step) in zip(pairs, extra):
        p.meta["radius"] = radius
        p.meta["step"] = step
    return pairs


def _serve_pair(args):
    side, dtype_name, kind, params, seed = args
    return speckle_pair((side, side), int(round(24000 * (side / 2048.0) ** 2)), Field(kind, params), 1.0, seed,
                        dtype=np.dtype(dtype_name).type)


def serve_workload(n_requests: int = 40, rate: float = 40.0, seed: int = BASE_SEED + 3,
                   sides=(1024, 2048, 3072, 4096), pool=None):
    """Served request stream: Poisson arrivals at ``rate`` per second, sides uniform over
    ``sides``, uint8 or uint16, a Gaussian bump (3 px, sigma = side / 6) or an affine field
    (translation U(-5, 5), gradients U(-0.01, 0.01)), radius in {7, 11, 15, 21, 25} and POI step
    in {3, 5, 8}.  Returns [(arrival seconds from the start, Pair)]; pairs render in ``pool``
    when one is given."""
    rng = np.random.default_rng(seed)
    specs, extra, t = [], [], 0.0
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        side = int(rng.choice(sides))
        dtype = np.uint8 if rng.uniform() < 0.5 else np.uint16
        if rng.uniform() < 0.5:
            kind = "bump"
            params = dict(cx=side / 2.0, cy=side / 2.0, s=side / 6.0, a=3.0, shear=0.0, sa=0.0, sl=64.0)
        else:
            kind = "linear"
            params = dict(u0=rng.uniform(-5, 5), ux=rng.uniform(-0.01, 0.01), uy=rng.uniform(-0.01, 0.01),
                          v0=rng.uniform(-5, 5), vx=rng.uniform(-0.01, 0.01), vy=rng.uniform(-0.01, 0.01))
            params["u0"] -= params["ux"] * side / 2 + params["uy"] * side / 2
            params["v0"] -= params["vx"] * side / 2 + params["vy"] * side / 2
        radius = int(rng.choice([7, 11, 15, 21, 25]))
        step = int(rng.choice([3, 5, 8]))
        specs.append((side, np.dtype(dtype).name, kind, params, seed * 1000 + i))
        extra.append((t, radius, step, kind))
    pairs = list(pool.map(_serve_pair, specs)) if pool is not None else [_serve_pair(a) for a in specs]
    out = []
    for p, (arrival, radius, step, kind) in zip(pairs, extra):
        p.meta.update(radius=radius, step=step, kind=kind)
        out.append((arrival, p))
    return out
