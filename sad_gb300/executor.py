"""Many fits and renders in flight on one GPU (the C executor of include/sad_gb300.h).

    with Executor(workers=8) as ex:
        f = ex.submit_fit(image, n_sites=4096, iterations=2000)   # image [H,W,3] f32 in [0,1]
        r = ex.submit_render(sites, 1024, 1024)                   # sites [N,10] f32
        sites, psnr = f.result()
        rgb = r.result()

Resident fits: `s = ex.open_fit(image, ...)`, then `s.continue_fit(k)` requests (more
iterations of the same fit, its state kept on the device), then `s.close()`.

The executor holds every request (and so the host arrays its worker reads and writes)
until the request completes, whether or not the caller keeps it.  Results are bitwise those
of a single fit (sad_trainer_fit_host) or render (sad_render_from_sites) of the same input.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class RequestError(RuntimeError):
    pass


class _Request:
    def __init__(self, ex: "Executor", kind: str, keep: tuple, out: np.ndarray):
        self._ex = ex
        self.kind = kind
        self._keep = keep  # host arrays the worker reads or writes
        self._out = out
        self.res = _lib.RequestResult()
        self.ticket = C.c_uint64(0)
        self._done = False

    def wait(self) -> "_Request":
        if not self._done:
            self._ex._check(self._ex._lib.sad_executor_wait(self._ex._h, self.ticket))
            self._done = True
            self._ex._pending.pop(self.ticket.value, None)
        if self.res.status != 0:
            raise RequestError(self.res.message.decode(errors="replace"))
        return self

    @property
    def queue_ms(self) -> float:
        return self.res.queue_ms

    @property
    def run_ms(self) -> float:
        return self.res.run_ms

    def result(self):
        self.wait()
        if self.kind == "fit":
            return self._out[: self.res.sites_written].copy(), float(self.res.psnr)
        if self.kind == "continue":
            return self._out[: self.res.sites_written].copy(), float(self.res.psnr), int(self.res.iteration)
        if self.kind in ("open", "close"):
            return float(self.res.psnr)
        return self._out


class FitSession:
    """A resident fit (sad_executor_open_fit): its sites, Adam moments and candidate fields
    stay on the device between continue() requests, until close()."""

    def __init__(self, ex: "Executor", session: int, opened: _Request, capacity: int):
        self._ex = ex
        self.id = session
        self.opened = opened
        self._capacity = capacity
        self.closed = False

    def continue_fit(self, iterations: int, sites: bool = True) -> _Request:
        """Queue `iterations` more iterations; result() gives (active sites, PSNR, iterations
        run so far)."""
        cap = self._capacity if sites else 0
        out = np.zeros((max(cap, 1), 10), np.float32)
        req = _Request(self._ex, "continue", (), out)
        self._ex._check(self._ex._lib.sad_executor_submit_continue(
            self._ex._h, self.id, int(iterations), out.ctypes.data_as(C.c_void_p), cap, C.byref(req.res),
            C.byref(req.ticket)))
        self._ex._pending[req.ticket.value] = req
        return req

    def close(self) -> _Request:
        req = _Request(self._ex, "close", (), np.zeros(0, np.float32))
        self._ex._check(self._ex._lib.sad_executor_close_fit(self._ex._h, self.id, C.byref(req.res),
                                                             C.byref(req.ticket)))
        self._ex._pending[req.ticket.value] = req
        self.closed = True
        return req


class Executor:
    def __init__(self, workers: int = 8, hbm_budget_bytes: int = 0, max_running_fits: int = 0):
        self._lib = _lib.load()
        cfg = _lib.ExecutorConfig()
        self._lib.sad_executor_config_default(C.byref(cfg))
        cfg.workers = workers
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.max_running_fits = max_running_fits
        self._h = C.c_void_p()
        self._pending: dict[int, _Request] = {}  # submitted, not yet waited for
        self._check(self._lib.sad_executor_create(C.byref(cfg), C.byref(self._h)))

    def _check(self, status: int) -> None:
        if status != 0:
            raise RuntimeError(self._lib.sad_last_error().decode(errors="replace"))

    def submit_fit(self, image: np.ndarray, mask: np.ndarray | None = None,
                   config: _lib.TrainConfig | None = None, **overrides) -> _Request:
        img = np.ascontiguousarray(image, dtype=np.float32)
        h, w = img.shape[:2]
        cfg = config if config is not None else _lib.TrainConfig()
        if config is None:
            self._lib.sad_train_config_default(C.byref(cfg))
            cfg.log_freq = 0
        for k, v in overrides.items():
            setattr(cfg, k, v)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        cap = max(cfg.max_sites, cfg.n_sites, 2 * w * h)  # bounds the trainer's site buffer
        out = np.zeros((cap, 10), np.float32)
        req = _Request(self, "fit", (img, m, cfg), out)
        self._check(self._lib.sad_executor_submit_fit(
            self._h, C.byref(cfg), img.ctypes.data_as(C.c_void_p),
            None if m is None else m.ctypes.data_as(C.c_void_p), w, h,
            out.ctypes.data_as(C.c_void_p), cap, C.byref(req.res), C.byref(req.ticket)))
        self._pending[req.ticket.value] = req
        return req

    def open_fit(self, image: np.ndarray, mask: np.ndarray | None = None,
                 config: _lib.TrainConfig | None = None, **overrides) -> FitSession:
        """Start a resident fit session (target up, init); see FitSession."""
        img = np.ascontiguousarray(image, dtype=np.float32)
        h, w = img.shape[:2]
        cfg = config if config is not None else _lib.TrainConfig()
        if config is None:
            self._lib.sad_train_config_default(C.byref(cfg))
            cfg.log_freq = 0
        for k, v in overrides.items():
            setattr(cfg, k, v)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        req = _Request(self, "open", (img, m, cfg), np.zeros(0, np.float32))
        sid = C.c_uint64(0)
        self._check(self._lib.sad_executor_open_fit(
            self._h, C.byref(cfg), img.ctypes.data_as(C.c_void_p),
            None if m is None else m.ctypes.data_as(C.c_void_p), w, h, C.byref(req.res), C.byref(sid),
            C.byref(req.ticket)))
        self._pending[req.ticket.value] = req
        return FitSession(self, sid.value, req, max(cfg.max_sites, cfg.n_sites, 2 * w * h))

    def submit_render(self, sites: np.ndarray, width: int, height: int,
                      config: _lib.RenderConfig | None = None) -> _Request:
        s = np.ascontiguousarray(sites, dtype=np.float32)
        cfg = config if config is not None else _lib.RenderConfig()
        if config is None:
            self._lib.sad_render_config_default(C.byref(cfg))
        out = np.zeros((height, width, 3), np.float32)
        req = _Request(self, "render", (s, cfg), out)
        self._check(self._lib.sad_executor_submit_render(
            self._h, C.byref(cfg), s.ctypes.data_as(C.c_void_p), s.shape[0], width, height,
            out.ctypes.data_as(C.c_void_p), C.byref(req.res), C.byref(req.ticket)))
        self._pending[req.ticket.value] = req
        return req

    def cancel(self, req: _Request) -> bool:
        """Withdraw a request that has not started (True); one that has started or finished
        completes as submitted (False).  A withdrawn request's result() raises RequestError."""
        flag = C.c_int(0)
        self._check(self._lib.sad_executor_cancel(self._h, req.ticket, C.byref(flag)))
        if flag.value:
            req._done = True
            self._pending.pop(req.ticket.value, None)
        return bool(flag.value)

    def inject_slab_failures(self, count: int) -> None:
        """Failure testing: refuse the next `count` slab allocations on the host (no GPU fault)."""
        self._check(self._lib.sad_executor_inject_slab_failures(self._h, count))

    def wait_all(self) -> None:
        self._check(self._lib.sad_executor_wait_all(self._h))
        for req in self._pending.values():
            req._done = True
        self._pending.clear()

    def close(self) -> None:
        if self._h:
            self._lib.sad_executor_destroy(self._h)  # runs what is queued, then joins
            self._h = C.c_void_p()
            for req in self._pending.values():
                req._done = True
            self._pending.clear()

    def __del__(self):
        self.close()

    def __enter__(self) -> "Executor":
        return self

    def __exit__(self, *exc) -> None:
        self.close()
