"""Host side of the serving loop, without a device: a bad request is refused at submission (as
subset.compute refuses it), so the loop never meets it; a good one is queued.  The admission and
batching loop itself runs on its host thread with the device steps replaced: requests are batched,
one that fails its preparation fails alone, and an error outside any request (a device fault)
fails every pending request and ends the loop instead of leaving them waiting."""
import collections
import threading

import numpy as np
import pytest


def _bare_server():
    from traditional_dic_gb300 import serve
    srv = serve.Server.__new__(serve.Server)   # no device: only the submission state
    srv._cv = threading.Condition()
    srv._queue = collections.deque()
    srv._next_id = 0
    srv._stop = False
    return srv


def test_submit_refuses_bad_requests(pkg):
    srv = _bare_server()
    img = np.zeros((32, 32), np.float32)
    with pytest.raises(RuntimeError, match="config must be a dict"):
        srv.submit(img, img, config="x.yaml")
    with pytest.raises(RuntimeError):
        srv.submit(img, img, config={"optimization": {"method": "lm"}})
    with pytest.raises(RuntimeError, match="2D numpy array"):
        srv.submit(np.zeros((4, 4, 3), np.float32), img)
    assert not srv._queue
    req = srv.submit(img, img, config={"subset": {"radius": 7}})
    assert list(srv._queue) == [req] and req.id == 0 and not req._done.is_set()


def test_footprint_counts_images_coefficients_and_grid(pkg):
    from traditional_dic_gb300 import serve, subset as S
    cfg = S.config_from_dict({"reliability_propagation": {"spacing": 4}})
    small = serve._footprint(100, 80, cfg)
    assert small > 2 * 4 * 100 * 80 + 260 * 20 * 16
    cfg.precision = 1
    assert serve._footprint(100, 80, cfg) > small   # FP64 coefficients


class _Event:
    def __init__(self, fail):
        self.fail = fail

    def query(self):
        if self.fail:
            raise RuntimeError("device fault")
        return True


class _Pair:
    made = 0
    closed = 0

    def __init__(self):
        _Pair.made += 1

    def close(self):
        _Pair.closed += 1


def _looping_server(fail_query=False):
    """The real admission / batching loop on a host thread, with the device steps replaced:
    preparation fails for a pair whose first pixel is -1, a batch finishes at once (or its
    completion query raises, as a device fault would)."""
    import time
    from traditional_dic_gb300 import serve
    srv = _bare_server()
    srv.memory_budget, srv.max_batch, srv._stop, srv._held = 1 << 40, 3, False, 0
    srv.batches, srv.stats = [], {"prepare": [], "propagate": [], "collect": []}

    def prepare(req):
        req.started = time.perf_counter()
        if req.reference[0, 0] == -1:
            raise ValueError("bad pair")
        return serve._Prepared(req, _Pair(), None, None, 1)

    def launch(ready):
        group, rest = ready[:srv.max_batch], ready[srv.max_batch:]
        srv.batches.append(len(group))
        return (None, group, _Event(fail_query), None), rest

    def collect(inflight):
        for p in inflight[1]:
            srv._complete(p.req, {"id": p.req.id, "batch": len(inflight[1])})
            p.pair.close()
            srv._held -= p.bytes

    srv._prepare, srv._launch, srv._collect = prepare, launch, collect
    srv._thread = threading.Thread(target=srv._loop, daemon=True)
    return srv


def test_loop_batches_requests_and_isolates_a_failing_one(pkg):
    srv = _looping_server()
    imgs = [np.full((16, 16), -1.0 if i == 4 else float(i), np.float32) for i in range(10)]
    reqs = [srv.submit(im, im) for im in imgs]
    srv._thread.start()
    for i, r in enumerate(reqs):
        if i == 4:
            with pytest.raises(ValueError, match="bad pair"):
                r.wait(10)
        else:
            assert r.wait(10)["id"] == i
    assert sum(srv.batches) == 9 and max(srv.batches) <= 3 and srv._held == 0
    srv.close()
    assert not srv._thread.is_alive()
    with pytest.raises(RuntimeError, match="closed"):
        srv.submit(imgs[0], imgs[0])


def test_loop_fails_every_pending_request_on_a_device_error(pkg):
    srv = _looping_server(fail_query=True)
    img = np.ones((16, 16), np.float32)
    made, closed = _Pair.made, _Pair.closed
    reqs = [srv.submit(img, img) for _ in range(7)]
    srv._thread.start()
    for r in reqs:
        with pytest.raises(RuntimeError, match="device fault"):
            r.wait(10)
    srv._thread.join(10)
    assert not srv._thread.is_alive()
    # the prepared pairs and those of the batch in flight are released, the budget with them
    assert _Pair.made - made > 0 and _Pair.closed - closed == _Pair.made - made
    assert srv._held == 0
    with pytest.raises(RuntimeError, match="closed"):
        srv.submit(img, img)


def test_submit_takes_a_config_structure_by_copy(pkg):
    from traditional_dic_gb300 import _lib as L
    srv = _bare_server()
    img = np.zeros((32, 32), np.float32)
    cfg = L.default_config()
    cfg.truncate_roi_subsets = 1
    req = srv.submit(img, img, config=cfg)
    cfg.subset_radius = 3                                   # the caller's later change stays theirs
    assert isinstance(req.config, L.Config) and req.config.truncate_roi_subsets == 1
    assert req.config.subset_radius == L.default_config().subset_radius


def test_masked_footprint_counts_the_padded_pair(pkg):
    from traditional_dic_gb300 import serve, subset as S
    cfg = S.config_from_dict({"reliability_propagation": {"spacing": 4}})
    plain = serve._footprint(100, 80, cfg)
    cfg.truncate_roi_subsets = 1
    pad = S.padding(cfg)
    assert pad > 0
    assert serve._footprint(100, 80, cfg) == serve._footprint(100 + 2 * pad, 80 + 2 * pad, S.config_from_dict(
        {"reliability_propagation": {"spacing": 4}})) > plain


@pytest.mark.parametrize("shape,radius,spacing", [((100, 80), 15, 4), ((64, 97), 7, 2), ((33, 50), 21, 9)])
def test_padded_roi_and_crop_give_the_truncated_grid(pkg, oracle, shape, radius, spacing):
    """The serving loop's masked collection: the padded pair's grid (gx * step, gy * step over the
    padded image) cropped to the image and shifted back is the truncated grid of
    SubsetDIC::compute (the oracle's dimensions, row-major, x = gx * step - pad)."""
    from traditional_dic_gb300 import _lib as L, subset as S
    h, w = shape
    cfg = L.default_config()
    cfg.subset_radius, cfg.propagation_spacing, cfg.truncate_roi_subsets = radius, spacing, 1
    pad = S.padding(cfg)
    assert pad == oracle.subset_padding(cfg)
    roi = np.zeros(shape, bool)
    roi[5:, 3:] = True
    proi = S.padded_roi(roi, w, h, pad)
    assert proi.shape == (h + 2 * pad, w + 2 * pad) and proi.sum() == roi.sum()
    assert np.array_equal(proi[pad:pad + h, pad:pad + w], roi)
    assert S.padded_roi(None, w, h, pad).sum() == w * h
    step = spacing + 1
    pgw, pgh = L.grid_dims(w + 2 * pad, h + 2 * pad, spacing)
    gy, gx = np.divmod(np.arange(pgw * pgh), pgw)
    padded = {"x": (gx * step).astype(np.float64), "y": (gy * step).astype(np.float64),
              "u": np.arange(pgw * pgh, dtype=np.float64), "valid": (gx % 2).astype(bool)}
    got = S.crop_padded(padded, w, h, pad)
    gw, gh = oracle.truncated_grid_dims(w, h, cfg)
    assert (gw, gh) == L.subset_grid_dims(w, h, cfg)
    assert len(got["x"]) == gw * gh
    xs = np.unique(got["x"])
    ys = np.unique(got["y"])
    assert len(xs) == gw and len(ys) == gh
    assert xs[0] == (-pad) % step and ys[0] == (-pad) % step and xs[-1] < w and ys[-1] < h
    assert np.array_equal(got["x"], np.tile(xs, gh)) and np.array_equal(got["y"], np.repeat(ys, gw))
    keep = got["u"].astype(int)                             # the rows kept, in grid order
    assert np.all(np.diff(keep) > 0)
    assert np.array_equal(got["valid"], padded["valid"][keep])
