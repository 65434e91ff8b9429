"""Result files of the subset workflow, mirroring python/traditional_dic/workflows/subset_2d.py:
the displacement CSV (save_subset_csv, :34-54) and the statistics JSON (write_stats, :94-113),
written from a result dict of ``subset.compute`` (host arrays) or of a batch job."""
from __future__ import annotations

import csv
import json
from pathlib import Path

import numpy as np

SUBSET_COLUMNS = ["x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "valid"]


def save_subset_csv(result: dict, path) -> None:
    """One row per grid point: x, y, u, v, the four displacement gradients, correlation, valid."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    cols = [np.asarray(result[k]) for k in SUBSET_COLUMNS]
    with path.open("w", newline="", encoding="utf-8") as f:
        writer = csv.writer(f)
        writer.writerow(SUBSET_COLUMNS)
        for i in range(len(cols[0])):
            writer.writerow([float(c[i]) for c in cols[:-1]] + [int(cols[-1][i])])


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
