"""Least-squares strain on the GPU, mirroring traditional_dic.postprocess
(python/traditional_dic/postprocess.py:13-28) and the binding
_traditional_dic.postprocess.compute_least_squares_strain_2d (bindings/python/bind_postprocess.cpp:44-46)."""
from __future__ import annotations

import csv
import ctypes as C
from pathlib import Path

import numpy as np

from . import _lib as L
from . import subset as S

STRAIN_FIELDS = ("du_dx", "du_dy", "dv_dx", "dv_dy", "exx", "eyy", "exy", "sample_count", "valid")


def compute_least_squares_strain_2d(points, displacement, radius, min_samples=6, green_lagrange=True, *,
                                    context: S.Context | None = None) -> np.recarray:
    """Per point: the plane fit of u and v over the points within ``radius`` (dic::
    compute_least_squares_strain_2d).  Returns a record array with the fields of
    dic::LeastSquaresStrain2D (``r[i].du_dx``, ``r.exx``, ...)."""
    pts = np.ascontiguousarray(points, np.float64)
    dsp = np.ascontiguousarray(displacement, np.float64)
    if pts.ndim != 2 or dsp.ndim != 2 or pts.shape[1] != 2 or dsp.shape[1] != 2 or pts.shape[0] != dsp.shape[0]:
        raise ValueError("points and displacement must both be Nx2 matrices")
    ctx = context or S.default_context()
    n = pts.shape[0]
    out = (L.LsStrain * max(n, 1))()
    ctx.check(ctx.lib.tdic_ls_strain_2d(ctx.handle, pts.ctypes.data, dsp.ctypes.data, n, float(radius),
                                        int(min_samples), int(bool(green_lagrange)), out, None))
    raw = np.ctypeslib.as_array(out)[:n]
    rec = np.zeros(n, dtype=[(f, np.float64) for f in STRAIN_FIELDS[:7]] + [("sample_count", np.int32),
                                                                               ("valid", np.bool_)])
    for f in STRAIN_FIELDS[:7]:
        rec[f] = raw[f]
    rec["sample_count"] = raw["sample_count"]
    rec["valid"] = raw["valid"] != 0
    return rec.view(np.recarray)


def save_least_squares_strain_csv(path, points, displacement, *, radius=None, elements=None, min_samples=6,
                                  green_lagrange=True, context: S.Context | None = None) -> None:
    """Write the least-squares strain of the points as CSV (header and row format of the
    reference's save_least_squares_strain_csv).  The finite-element variant (``elements``) is
    not on this path."""
    if elements is not None:
        raise NotImplementedError("mesh least-squares strain is not on the GPU path")
    if radius is None:
        raise ValueError("radius is required for subset least-squares strain")
    points = np.asarray(points, dtype=np.float64)
    strains = compute_least_squares_strain_2d(points, displacement, radius, min_samples, green_lagrange,
                                              context=context)
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    with path.open("w", newline="", encoding="utf-8") as f:
        writer = csv.writer(f)
        writer.writerow(["x", "y", "du_dx", "du_dy", "dv_dx", "dv_dy", "exx", "eyy", "exy", "sample_count", "valid"])
        for point, s in zip(points, strains):
            writer.writerow([point[0], point[1], float(s.du_dx), float(s.du_dy), float(s.dv_dx), float(s.dv_dy),
                             float(s.exx), float(s.eyy), float(s.exy), int(s.sample_count), int(s.valid)])
