"""Host side of the serving loop, without a device: a bad request is refused at submission (as
subset.compute refuses it), so the loop never meets it; a good one is queued."""
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
