"""Serving loop for streams of image pairs (continuous batching on one GPU).

Requests (``Server.submit``) arrive at any time.  A host thread admits them while their device
footprint fits the memory budget, prepares each on a preparation stream (upload, B-spline
prefilter, seed selection: ``SubsetDIC::compute``'s steps before the propagation), and
propagates all prepared requests in one batched persistent launch (``subset.Batch``) on the
propagation stream.  Requests that arrive while a batch is on the GPU are prepared meanwhile
and go into the next batch, so preparation kernels overlap the running propagation.  Each
request's result equals ``subset.compute`` of the same pair and configuration alone (the batch
gives every job the single-pair result).  A request with a full ``Config`` structure and masked
subsets (``truncate_roi_subsets``) is prepared as the padded pair, propagated with the padded ROI
in a batch of masked requests, and its grid cropped back: ``subset.compute_config``'s result.

Device memory comes from the context's caching pool, so the loop allocates none once warm.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import subset as S


@dataclass
class Request:
    """One submitted pair.  ``wait()`` returns the result dict of ``subset.compute``."""
    id: int
    reference: np.ndarray
    deformed: np.ndarray
    config: dict | None
    roi: np.ndarray | None
    arrival: float
    started: float = 0.0
    finished: float = 0.0
    batch_size: int = 0
    result: dict | None = None
    error: BaseException | None = None
    _done: threading.Event = field(default_factory=threading.Event, repr=False)

    def wait(self, timeout: float | None = None) -> dict:
        if not self._done.wait(timeout):
            raise TimeoutError(f"request {self.id} not finished")
        if self.error is not None:
            raise self.error
        return self.result

    @property
    def latency(self) -> float:
        """Seconds from submission to result."""
        return self.finished - self.arrival


@dataclass
class _Prepared:
    req: Request
    pair: S.Pair
    cfg: L.Config
    seed: L.Seed
    bytes: int
    roi: np.ndarray | None = None   # the ROI of the propagation (the padded pair's, masked subsets)
    pad: int = 0                    # masked subsets: the padding of the pair's images


def _config(config) -> L.Config:
    """The request's configuration: a config dict (``subset.compute``) or a full ``Config``
    structure (``subset.compute_config``, e.g. masked subsets); a copy either way."""
    if isinstance(config, L.Config):
        return L.Config.from_buffer_copy(config)
    return S.config_from_dict(config)


def _footprint(w: int, h: int, cfg: L.Config) -> int:
    """Device bytes of one request: its pair (float32 images, coefficients, upload staging) and
    the propagation scratch and outputs of its grid points (masked subsets: of the padded pair,
    with its pixel ROI)."""
    if cfg.truncate_roi_subsets:
        pad = S.padding(cfg)
        w, h = w + 2 * pad, h + 2 * pad
    gw, gh = L.grid_dims(w, h, cfg.propagation_spacing)
    coef = 8 if cfg.precision == L.FP64 else 4
    return 2 * 4 * w * h + coef * (w + 8) * (h + 8) + 8 * w * h + 260 * gw * gh


class Server:
    """Continuous-batching request loop on one device (see the module docstring).

    memory_budget: device bytes the admitted (prepared or running) requests may hold.
    max_batch: requests per batched launch (at most 512).
    reserve_sms: SMs the propagation leaves to the preparation of the next requests (the
    propagation holds its SMs until it ends; default a tenth of the device)."""

    def __init__(self, context: S.Context | None = None, memory_budget: int = 48 << 30, max_batch: int = 64,
                 reserve_sms: int | None = None):
        import torch
        self.ctx = context or S.default_context()
        self.memory_budget = int(memory_budget)
        self.max_batch = max(1, min(512, int(max_batch)))
        n_sms = torch.cuda.get_device_properties(self.ctx.device).multi_processor_count
        reserve = max(1, n_sms // 10) if reserve_sms is None else max(0, int(reserve_sms))
        self._sms = max(1, n_sms - reserve)
        self._torch = torch
        self._prep = torch.cuda.Stream()   # uploads, prefilter, seed selection
        self._main = torch.cuda.Stream()   # batched propagation
        self._copy = torch.cuda.Stream()   # results of finished batches to host
        self._queue: collections.deque[Request] = collections.deque()
        self._cv = threading.Condition()
        self._stop = False
        self._next_id = 0
        self._held = 0
        self.batches: list[int] = []  # size of every batch launched
        # seconds per request (preparation) and per batch (device propagation, collection of
        # the results to host arrays)
        self.stats: dict[str, list[float]] = {"prepare": [], "propagate": [], "collect": []}
        self._thread = threading.Thread(target=self._loop, name="tdic-serve", daemon=True)
        self._thread.start()

    # ---- client side -------------------------------------------------------------------------
    def submit(self, reference: np.ndarray, deformed: np.ndarray, config: dict | L.Config | None = None,
               roi=None) -> Request:
        """Queue one pair.  Bad images or a bad config dict raise here, as ``subset.compute``
        would.  ``config`` is a config dict, or a full ``Config`` structure as
        ``subset.compute_config`` takes (the result is then ``compute_config``'s, e.g. with
        masked subsets); a structure's values are checked when the request is prepared, and a
        bad one fails that request alone."""
        ref = S._check_image(reference, "reference")
        de = S._check_image(deformed, "deformed")
        if config is not None and not isinstance(config, (dict, L.Config)):
            raise RuntimeError("config must be a dict (from YAML) or None.")
        if isinstance(config, L.Config):
            config = L.Config.from_buffer_copy(config)   # the caller may change theirs meanwhile
        _config(config)
        with self._cv:
            if self._stop:
                raise RuntimeError("the server is closed")
            req = Request(self._next_id, ref, de, config, roi, time.perf_counter())
            self._next_id += 1
            self._queue.append(req)
            self._cv.notify()
        return req

    def close(self) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify()
        self._thread.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- server side -------------------------------------------------------------------------
    def _prepare(self, req: Request) -> _Prepared | None:
        """Upload, prefilter and seed selection on the preparation stream.  None when the
        request finished here (no seed: the reference's empty result)."""
        req.started = time.perf_counter()
        cfg = _config(req.config)
        cfg.propagation_mode = S.PROPAGATION_MODES["dataflow"]
        h, w = req.reference.shape
        if req.roi is not None and np.asarray(req.roi).shape != (h, w):
            self._complete(req, S._empty_result())
            return None
        pair, seed = S.prepare(self.ctx, req.reference, req.deformed, cfg, roi=req.roi, stream=self._prep)
        self.stats["prepare"].append(time.perf_counter() - req.started)
        if not seed.found:
            pair.close()
            self._complete(req, S._empty_result())
            return None
        if cfg.truncate_roi_subsets:   # the padded pair: its ROI, and the crop at collection
            pad = S.padding(cfg)
            return _Prepared(req, pair, cfg, seed, _footprint(w, h, cfg), S.padded_roi(req.roi, w, h, pad), pad)
        return _Prepared(req, pair, cfg, seed, _footprint(w, h, cfg), req.roi)

    def _complete(self, req: Request, result=None, error=None) -> None:
        req.result, req.error = result, error
        req.finished = time.perf_counter()
        req._done.set()

    def _launch(self, ready: list[_Prepared]):
        first = ready[0]
        def sig(p):   # what every job of one batched launch shares
            return p.pair.degree, p.pair.precision, p.cfg.optimizer, p.cfg.truncate_roi_subsets != 0

        group = [p for p in ready if sig(p) == sig(first)][:self.max_batch]
        rest = [p for p in ready if p not in group]
        self._prep.synchronize()  # the group's pairs and seeds are ready
        batch = S.Batch(self.ctx, [p.pair for p in group], [p.cfg for p in group], [p.seed for p in group],
                        [p.roi for p in group], stream=self._main)
        batch.set_sms(self._sms)
        start = self._torch.cuda.Event(enable_timing=True)
        done = self._torch.cuda.Event(enable_timing=True)
        start.record(self._main)
        batch.launch(stream=self._main)
        done.record(self._main)
        self.batches.append(len(group))
        return (batch, group, done, start), rest

    def _collect(self, inflight) -> None:
        batch, group, done, start = inflight
        t0 = time.perf_counter()
        self.stats["propagate"].append(start.elapsed_time(done) / 1e3)
        try:
            pc = batch.finish(stream=self._copy)
            for j, p in enumerate(group):
                p.req.batch_size = len(group)
                if pc[j] == 0:
                    self._complete(p.req, S._empty_result())
                else:
                    out = batch.outputs(j, stream=self._copy)
                    res = {k: out[k] for k in S.RESULT_KEYS + S.EXTRA_KEYS}
                    if p.cfg.truncate_roi_subsets:
                        h, w = p.req.reference.shape
                        res = S.crop_padded(res, w, h, p.pad)
                    self._complete(p.req, res)
        except BaseException as exc:  # every request of the batch learns of the failure
            for p in group:
                if not p.req._done.is_set():
                    self._complete(p.req, error=exc)
        finally:
            batch.close()
            for p in group:
                p.pair.close()
                self._held -= p.bytes
            self.stats["collect"].append(time.perf_counter() - t0)

    def _loop(self) -> None:
        inflight = None
        ready: list[_Prepared] = []
        try:
            while True:
                with self._cv:
                    if self._stop and not self._queue and not ready and inflight is None:
                        break
                    if not self._queue and not ready and inflight is None:
                        self._cv.wait(0.05)
                        continue
                progressed = False
                finished = None
                if inflight is not None and inflight[2].query():
                    finished, inflight = inflight, None
                    progressed = True
                # the next batch goes to the GPU first; the finished one's results are copied out
                # (on the copy stream) while it runs
                if inflight is None and ready:
                    try:
                        inflight, ready = self._launch(ready)
                    except BaseException as exc:
                        for p in ready:
                            self._complete(p.req, error=exc)
                            p.pair.close()
                            self._held -= p.bytes
                        ready = []
                    progressed = True
                if finished is not None:
                    self._collect(finished)
                # admit and prepare queued requests while the budget allows (overlaps the batch)
                while len(ready) < self.max_batch:
                    with self._cv:
                        if not self._queue:
                            break
                        req = self._queue[0]
                        h, w = req.reference.shape
                        try:
                            est = _footprint(w, h, _config(req.config))
                        except Exception:
                            est = 0  # _prepare raises the same error and fails this request alone
                        if self._held + est > self.memory_budget and (ready or inflight is not None):
                            break  # wait for memory to free up
                        self._queue.popleft()
                    try:
                        prepared = self._prepare(req)
                    except BaseException as exc:
                        self._complete(req, error=exc)
                        prepared = None
                    progressed = True
                    if prepared is not None:
                        self._held += prepared.bytes
                        ready.append(prepared)
                    if inflight is not None and inflight[2].query():
                        break  # launch the next batch without delay
                if not progressed:
                    time.sleep(0.0002)
        except BaseException as exc:  # an error outside any one request (a device fault): fail them all
            self._fail_pending(exc, ready, inflight)

    def _fail_pending(self, exc: BaseException, ready, inflight) -> None:
        """Fail every request not yet answered and release what they hold on the device: the
        prepared pairs, the batch in flight and its pairs (each release on its own, so one that
        fails does not keep the others)."""
        with self._cv:
            self._stop = True
            pending = list(self._queue)
            self._queue.clear()
        held = list(ready)
        if inflight is not None:
            held += list(inflight[1])
            try:
                inflight[0].close()
            except Exception:
                pass
        for p in held:
            pending.append(p.req)
            try:
                p.pair.close()
            except Exception:
                pass
        self._held = 0
        for req in pending:
            if not req._done.is_set():
                self._complete(req, error=exc)
