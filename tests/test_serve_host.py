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
