"""Python handle on the lockstep batch of fits (sad_batch_* of the C ABI).

    b = Batch([(w0, h0), (w1, h1), ...])          # training_config.json defaults
    for i, img in enumerate(images): b.set_target(i, img)
    b.init(); b.run()                              # every image, one launch per stage
    sites, psnr = b.sites(i), b.psnr(i)

Each image's result is bitwise the one its own Trainer fit gives; the batch runs every
stage of an iteration as one launch over all images.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .config import train_config
from .trainer import Trainer


class _ImageView(Trainer):
    """A batch image's trainer, owned by the batch (closing it does nothing)."""

    def __init__(self, handle: C.c_void_p, cfg, width: int, height: int):
        self.width, self.height = int(width), int(height)
        self.cfg = cfg
        self._h = handle

    def close(self) -> None:
        pass


class Batch:
    def __init__(self, sizes, config: _lib.TrainConfig | None = None, **overrides):
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        self.cfg = config if config is not None else train_config(**overrides)
        if config is not None:
            for k, v in overrides.items():
                setattr(self.cfg, k, v)
        n = len(self.sizes)
        ws = (C.c_int * n)(*[w for w, _ in self.sizes])
        hs = (C.c_int * n)(*[h for _, h in self.sizes])
        self._h = C.c_void_p()
        _lib.call("sad_batch_create", C.byref(self.cfg), n, ws, hs, C.byref(self._h))
        self.images = []
        for i, (w, h) in enumerate(self.sizes):
            t = C.c_void_p()
            _lib.call("sad_batch_trainer", self._h, i, C.byref(t))
            self.images.append(_ImageView(t, self.cfg, w, h))

    def close(self) -> None:
        if self._h:
            _lib.call("sad_batch_destroy", self._h)
            self._h = C.c_void_p()
            self.images = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_target(self, i: int, image, mask=None) -> None:
        self.images[i].set_target(image, mask)

    def init(self) -> None:
        _lib.call("sad_batch_init", self._h)

    def run(self, end: int | None = None) -> None:
        _lib.call("sad_batch_run", self._h, self.cfg.iterations if end is None else int(end))

    def synchronize(self) -> None:
        _lib.call("sad_batch_synchronize", self._h)

    def stream(self) -> int:
        return _lib.fn("sad_batch_stream")(self._h)

    def enable_timing(self, on: bool = True) -> None:
        _lib.call("sad_batch_enable_timing", self._h, int(on))

    def gradient_ms(self) -> float:
        v = C.c_double()
        _lib.call("sad_batch_gradient_ms", self._h, C.byref(v))
        return float(v.value)

    def psnr(self, i: int) -> float:
        return self.images[i].psnr()

    def sites(self, i: int, active_only: bool = True) -> np.ndarray:
        return self.images[i].sites(active_only)


def fit_batch(images, **overrides):
    """Fit every image of `images` (numpy [H,W,3] f32) in one lockstep batch; returns a
    list of (active sites, PSNR)."""
    with Batch([(im.shape[1], im.shape[0]) for im in images], **overrides) as b:
        for i, im in enumerate(images):
            b.set_target(i, im)
        b.init()
        b.run()
        b.synchronize()
        return [(b.sites(i), b.psnr(i)) for i in range(len(images))]
