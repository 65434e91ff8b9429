"""Result files of the subset workflow, mirroring python/traditional_dic/workflows/subset_2d.py:
the displacement CSV (save_subset_csv, :34-54) and the statistics JSON (write_stats, :94-113).

The CSV is written by the library (tdic_write_subset_csv): byte for byte the file the reference's
csv.writer loop writes, formatted on every host thread, from host arrays (a result dict of
``subset.compute``) or straight from device arrays (``save_subset_csv_device``: a batch job's or a
propagation's device outputs)."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

from . import _lib as L

SUBSET_COLUMNS = ["x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "valid"]


def save_subset_csv(result: dict, path, context=None) -> None:
    """One row per grid point: x, y, u, v, the four displacement gradients, correlation, valid."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    cols = {k: np.ascontiguousarray(result[k], dtype=np.float64) for k in SUBSET_COLUMNS[:-1]}
    cols["valid"] = np.ascontiguousarray(result["valid"], dtype=np.uint8)
    n = len(cols["x"])
    if any(len(c) != n for c in cols.values()):
        raise ValueError("result columns differ in length")
    g = L.GridOut(**{k: cols[k].ctypes.data for k in SUBSET_COLUMNS})
    lib = L.load()
    handle = context.handle if context is not None else None  # host arrays need no device
    L.check(lib.tdic_write_subset_csv(handle, str(path).encode(), C.byref(g), L.HOST, n), handle)


def save_subset_csv_device(grid: "L.GridOut", n: int, path, context=None) -> None:
    """The same file from device arrays (x .. correlation float64, valid uint8, n points)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    if context is None:
        from . import subset as S
        context = S.default_context()
    context.check(context.lib.tdic_write_subset_csv(context.handle, str(path).encode(), C.byref(grid), L.DEVICE,
                                                    int(n)))


def subset_stats(result: dict, metric: str = "znssd") -> dict:
    """The statistics of write_stats over the valid points."""
    valid = np.asarray(result["valid"], dtype=bool)
    u = np.asarray(result["u"], dtype=np.float64)[valid]
    v = np.asarray(result["v"], dtype=np.float64)[valid]
    q = np.asarray(result["correlation"], dtype=np.float64)[valid]
    mag = np.hypot(u, v)
    return {
        "total_points": int(len(result["x"])),
        "valid_points": int(np.sum(valid)),
        "invalid_points": int(len(result["x"]) - np.sum(valid)),
        "u_mean": float(u.mean()) if u.size else 0.0,
        "u_std": float(u.std()) if u.size else 0.0,
        "v_mean": float(v.mean()) if v.size else 0.0,
        "v_std": float(v.std()) if v.size else 0.0,
        "mag_mean": float(mag.mean()) if mag.size else 0.0,
        "mag_max": float(mag.max()) if mag.size else 0.0,
        f"{metric}_mean": float(q.mean()) if q.size else 0.0,
        f"{metric}_max": float(q.max()) if q.size else 0.0,
    }


def write_stats(result: dict, path, metric: str = "znssd") -> None:
    Path(path).write_text(json.dumps(subset_stats(result, metric), indent=2), encoding="utf-8")
