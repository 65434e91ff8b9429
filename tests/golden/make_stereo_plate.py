"""Generate tests/golden/stereo_plate_fields.npz: subset-DIC fields computed by the reference itself.

The reference checkout keeps three outputs of its own subset solver for the stereo plate case
(tests/data/f0b/stereo_plate/fields/{left_temporal,reference_disparity,deformed_disparity}.npz,
each with a JSON sidecar naming its inputs and configuration).  They were written by the stereo
workflow (python/traditional_dic/workflows/stereo_3d.py:167-185):

  * images read by ``read_gray`` (stereo_3d.py:34-40): PIL ``convert("F")`` of the 8-bit BMP,
    divided by the image's maximum, as float32;
  * the ROI by ``read_mask`` (stereo_3d.py:43-44): PIL ``convert("L")`` of ROI.bmp, > 0;
  * ``tdic.subset(reference, deformed, config=normalize_subset_config(config/subset_2d.yaml),
    roi=roi)`` -- the pybind dict parser sees the YAML's subset section as it stands: radius 41,
    50 iterations, threshold 1e-6, quintic B-spline (degree 5), first-order ZNSSD ICGN,
    propagation spacing 3 (stride 4), propagation max_znssd 2.0;
  * the result's x, y, u, v, correlation, valid written for every point of the 360 x 270 grid.

This script keeps what a rerun of that path needs, so that tests can run where the reference
checkout is absent:

  * a BMP reader for the case's files (uncompressed, 8 bits per pixel with a 256-entry palette,
    bottom-up rows padded to 4 bytes).  The three camera images carry the linear grey ramp
    palette, for which PIL opens them in mode "L" and ``convert("F")`` returns the palette
    index exactly; the ROI's palette maps index 0 to black and every other index used (255) to a
    non-zero grey, so ``convert("L") > 0`` is ``index != 0``.  The reader checks both facts;
  * a crop of the 1440 x 1080 images: the ROI's bounding box widened by the subset radius, the
    quintic stencil, the largest displacement in the stored fields and 48 px.  The B-spline
    prefilter is a recursive filter whose slowest pole is -0.4306 (degree 5), so the crop's own
    borders change coefficients at 48 px from them by a relative 0.43^48 ~ 3e-18: inside the
    margin the coefficients are the full image's.  The crop origin is a multiple of the grid
    stride (4), so the crop's grid points are grid points of the full image;
  * the images as uint8 crops and each full image's maximum (``read_gray`` divides by it);
  * per field the crop-grid index, u, v and correlation of every valid point (all invalid
    points hold zeros in the reference's output), and the seed the reference propagated from.

Seeds.  The reference seeded from SIFT matches (OpenCV), which this build does not have.  For
left_temporal the reference's seed point can be read off its output: grid point (852, 624) is
the only one whose stored result is not a propagation solve (its correlation 0.0243 is the
field's maximum, where every solve of that subset gives 0.00635), i.e. the refined seed stored
as it came (reliability_propagation.cpp:246-253, seed on a grid point).  Seeding there with the
stored u, v (displacement gradients zero, not stored) reproduces the reference's start.  For
reference_disparity no point stands out (the reference's seed was off the grid and solved again
there); the seed is placed one pixel off the grid point nearest the ROI centre with that point's
stored u, v, so it is solved again on the grid as the reference does.  At threshold 1e-6 and up
to 50 iterations every point converges strictly, and the converged result does not depend on
the visit order beyond the threshold.

Run from the repository root (needs the reference checkout):
    python tests/golden/make_stereo_plate.py
"""
import json
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "stereo_plate_fields.npz")
REF = "/root/reference"
CASE = os.path.join(REF, "case", "stereo_DIC", "plate_center_load")
FIELDS = os.path.join(REF, "tests", "data", "f0b", "stereo_plate", "fields")

STRIDE = 4           # reliability_propagation.spacing 3 -> stride 4
RADIUS = 41
MARGIN = 48          # px beyond subset + stencil + displacement: spline edge effect < 1e-17
FIELD_IMAGES = {"left_temporal": "cam1/04_L.bmp", "reference_disparity": "cam2/00_R.bmp"}
REFERENCE_IMAGE = "cam1/00_L.bmp"
# config/subset_2d.yaml as the pybind parser reads it (bind_subset.cpp:158-248)
CONFIG = {
    "subset": {"radius": 41},
    "shape_function": {"order": 1},
    "optimization": {"method": "icgn", "max_iterations": 50, "convergence_threshold": 1.0e-6},
    "correlation": {"criterion": "znssd"},
    "interpolation": {"method": "bspline", "degree": 5},
    "reliability_propagation": {"spacing": 3, "max_znssd": 2.0},
}


def read_bmp8(path):
    """Palette index image and palette (n x 4, B G R 0) of an uncompressed 8-bit BMP."""
    with open(path, "rb") as f:
        b = f.read()
    if b[:2] != b"BM":
        raise ValueError(f"{path}: not a BMP")
    data_off = struct.unpack_from("<I", b, 10)[0]
    hdr = struct.unpack_from("<I", b, 14)[0]
    w, h, planes, bpp, comp = struct.unpack_from("<iiHHI", b, 18)
    ncol = struct.unpack_from("<I", b, 46)[0] or 256
    if bpp != 8 or comp != 0 or planes != 1:
        raise ValueError(f"{path}: only uncompressed 8-bit BMPs are read")
    pal = np.frombuffer(b, np.uint8, count=4 * ncol, offset=14 + hdr).reshape(ncol, 4)
    stride = (w + 3) // 4 * 4
    rows = np.frombuffer(b, np.uint8, count=stride * abs(h), offset=data_off).reshape(abs(h), stride)[:, :w]
    img = rows[::-1] if h > 0 else rows          # positive height: bottom-up rows
    return np.ascontiguousarray(img), pal


def read_gray_u8(path):
    """The pixels PIL's convert("F") returns for the case's grey-ramp BMPs (as uint8)."""
    img, pal = read_bmp8(path)
    ramp = np.arange(len(pal), dtype=np.uint8)
    if not (np.array_equal(pal[:, 0], ramp) and np.array_equal(pal[:, 1], ramp) and np.array_equal(pal[:, 2], ramp)):
        raise ValueError(f"{path}: palette is not the grey ramp PIL opens as mode L")
    return img


def read_mask(path):
    """read_mask: convert("L") > 0, i.e. palette index of a non-black entry."""
    img, pal = read_bmp8(path)
    lum = (299 * pal[:, 2].astype(int) + 587 * pal[:, 1].astype(int) + 114 * pal[:, 0].astype(int)) // 1000
    if lum[0] != 0 or np.any(lum[np.unique(img)[1:]] == 0):
        raise ValueError(f"{path}: unexpected ROI palette")
    return (img != 0).astype(np.uint8)


def main():
    ref_full = read_gray_u8(os.path.join(CASE, REFERENCE_IMAGE))
    roi_full = read_mask(os.path.join(CASE, "ROI.bmp"))
    h, w = ref_full.shape
    gw, gh = -(-w // STRIDE), -(-h // STRIDE)
    ys, xs = np.nonzero(roi_full)
    fields, deformed = {}, {}
    umin = vmin = 0.0
    umax = vmax = 0.0
    for name, image in FIELD_IMAGES.items():
        z = np.load(os.path.join(FIELDS, name + ".npz"))
        side = json.load(open(os.path.join(FIELDS, name + ".json")))
        assert side["subset_config"] == "config/subset_2d.yaml" and side["solver"] == "subset"
        assert side["source_image_a"].endswith(REFERENCE_IMAGE) and side["source_image_b"].endswith(image)
        assert len(z["x"]) == gw * gh
        gx = np.arange(gw * gh) % gw
        gy = np.arange(gw * gh) // gw
        assert np.array_equal(z["x"], gx * STRIDE * 1.0) and np.array_equal(z["y"], gy * STRIDE * 1.0)
        valid = z["valid"].astype(bool)
        assert int(valid.sum()) == side["valid_count"]
        for k in ("u", "v", "correlation"):
            assert np.all(z[k][~valid] == 0.0)
        fields[name] = z
        deformed[name] = read_gray_u8(os.path.join(CASE, image))
        umin, umax = min(umin, z["u"][valid].min()), max(umax, z["u"][valid].max())
        vmin, vmax = min(vmin, z["v"][valid].min()), max(vmax, z["v"][valid].max())
    reach = RADIUS + 6 + MARGIN        # subset, quintic stencil (3) and a few px of warp growth, margin
    x0 = max(0, (xs.min() - reach + int(np.floor(umin))) // STRIDE * STRIDE)
    y0 = max(0, (ys.min() - reach + int(np.floor(vmin))) // STRIDE * STRIDE)
    x1 = min(w, xs.max() + reach + int(np.ceil(umax)) + 1)
    y1 = min(h, ys.max() + reach + int(np.ceil(vmax)) + 1)
    cw, ch = x1 - x0, y1 - y0
    cgw, cgh = -(-cw // STRIDE), -(-ch // STRIDE)
    # crop grid point (i % cgw, i // cgw) is full grid point (x0/4 + i % cgw, y0/4 + i // cgw)
    ci = np.arange(cgw * cgh)
    full = (y0 // STRIDE + ci // cgw) * gw + (x0 // STRIDE + ci % cgw)
    inside = ((ci % cgw) * STRIDE < cw) & ((ci // cgw) * STRIDE < ch)
    arrays = {
        "reference": ref_full[y0:y1, x0:x1].copy(),
        "reference_max": np.float32(ref_full.max()),
        "roi": roi_full[y0:y1, x0:x1].copy(),
        "origin": np.array([x0, y0], np.int64),
        "full_shape": np.array([h, w], np.int64),
        "config": np.array(json.dumps(CONFIG)),
    }
    cx, cy = (xs.min() + xs.max()) // 2, (ys.min() + ys.max()) // 2
    for name, z in fields.items():
        valid = z["valid"].astype(bool)
        # every valid point lies inside the crop's grid
        assert valid[full[inside]].sum() == valid.sum()
        keep = inside & valid[full]
        idx = ci[keep]
        arrays[f"{name}_deformed"] = deformed[name][y0:y1, x0:x1].copy()
        arrays[f"{name}_deformed_max"] = np.float32(deformed[name].max())
        arrays[f"{name}_index"] = idx.astype(np.int32)
        for k in ("u", "v", "correlation"):
            arrays[f"{name}_{k}"] = z[k][full[keep]].astype(np.float64)
        if name == "left_temporal":
            j = int(np.argmax(np.where(valid, z["correlation"], -1.0)))
            sx, sy = z["x"][j], z["y"][j]
            assert (sx, sy) == (852.0, 624.0)
        else:
            d2 = np.where(valid, (z["x"] - cx) ** 2 + (z["y"] - cy) ** 2, np.inf)
            j = int(np.argmin(d2))
            sx, sy = z["x"][j] + 1.0, z["y"][j]
        # seed in crop coordinates: x, y, u, v, correlation
        arrays[f"{name}_seed"] = np.array([sx - x0, sy - y0, z["u"][j], z["v"][j], z["correlation"][j]])
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: crop {cw} x {ch} at ({x0}, {y0}), grid {cgw} x {cgh}, "
          + ", ".join(f"{n}: {len(arrays[n + '_index'])} valid" for n in fields))


if __name__ == "__main__":
    main()
