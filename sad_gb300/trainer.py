"""Python handle on the device trainer (sad_trainer_* of the C ABI).

    tr = Trainer(width, height)                  # training_config.json defaults
    tr.set_target(image)                         # numpy [H,W,3] f32 or CUDA tensor
    tr.init()                                    # gradient-weighted sites
    tr.run()                                     # whole schedule (or run(end=k))
    psnr = tr.psnr(); sites = tr.sites()         # [K,10] active sites, device order
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .config import train_config


class Trainer:
    def __init__(self, width: int, height: int, config: _lib.TrainConfig | None = None,
                 **overrides):
        self.width, self.height = int(width), int(height)
        self.cfg = config if config is not None else train_config(**overrides)
        if config is not None:
            for k, v in overrides.items():
                setattr(self.cfg, k, v)
        self._h = C.c_void_p()
        _lib.call("sad_trainer_create", C.byref(self.cfg), self.width, self.height, C.byref(self._h))

    # -- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        if self._h:
            _lib.call("sad_trainer_destroy", self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- data --------------------------------------------------------------
    def set_target(self, image, mask=None) -> None:
        try:
            import torch
            is_tensor = isinstance(image, torch.Tensor)
        except ImportError:  # pragma: no cover
            is_tensor = False
        if is_tensor:
            image = image.contiguous()
            m = mask.contiguous() if mask is not None else None
            _lib.call("sad_trainer_set_target_device", self._h, C.c_void_p(image.data_ptr()),
                      C.c_void_p(m.data_ptr()) if m is not None else None)
            self._keep = (image, m)
        else:
            img = np.ascontiguousarray(image, dtype=np.float32)
            assert img.shape == (self.height, self.width, 3), img.shape
            m = np.ascontiguousarray(mask, dtype=np.float32) if mask is not None else None
            _lib.call("sad_trainer_set_target_host", self._h, img.ctypes.data_as(C.c_void_p),
                      m.ctypes.data_as(C.c_void_p) if m is not None else None)
            self._keep = (img, m)
            self.synchronize()

    def init(self, sites: np.ndarray | None = None) -> None:
        if sites is None:
            _lib.call("sad_trainer_init", self._h, None, 0)
        else:
            s = np.ascontiguousarray(sites, dtype=np.float32).reshape(-1, 10)
            _lib.call("sad_trainer_init", self._h, s.ctypes.data_as(C.c_void_p), s.shape[0])

    def run(self, end: int | None = None) -> None:
        _lib.call("sad_trainer_run", self._h, self.cfg.iterations if end is None else int(end))

    def synchronize(self) -> None:
        import torch
        stream = _lib.fn("sad_trainer_stream")(self._h)
        torch.cuda.ExternalStream(stream).synchronize()

    def render(self, out=None):
        """Render into a CUDA tensor [H,W,3] (allocated when `out` is None)."""
        import torch
        if out is None:
            out = torch.empty((self.height, self.width, 3), dtype=torch.float32, device="cuda")
        psnr = C.c_float()
        _lib.call("sad_trainer_render", self._h, C.c_void_p(out.data_ptr()), C.byref(psnr))
        return out

    def psnr(self) -> float:
        v = C.c_float()
        _lib.call("sad_trainer_render", self._h, None, C.byref(v))
        return float(v.value)

    def sites(self, active_only: bool = True) -> np.ndarray:
        info = self.info()
        out = np.empty((max(1, info.site_buffer), 10), dtype=np.float32)
        k = C.c_int()
        _lib.call("sad_trainer_get_sites", self._h, out.ctypes.data_as(C.c_void_p), out.shape[0],
                  int(active_only), C.byref(k))
        return out[: k.value].copy()

    def info(self) -> _lib.TrainerInfo:
        info = _lib.TrainerInfo()
        _lib.call("sad_trainer_info", self._h, C.byref(info))
        return info

    def enable_timing(self, on: bool = True) -> None:
        _lib.call("sad_trainer_enable_timing", self._h, int(on))

    def fit_host(self, image: np.ndarray, sites_out: np.ndarray | None = None):
        """One whole fit through the host-memory entry point; returns (sites, psnr)."""
        img = np.ascontiguousarray(image, dtype=np.float32)
        if sites_out is None:
            sites_out = np.empty((max(1, self.cfg.max_sites, self.cfg.n_sites), 10), dtype=np.float32)
        k, psnr = C.c_int(), C.c_float()
        _lib.call("sad_trainer_fit_host", self._h, img.ctypes.data_as(C.c_void_p), None,
                  sites_out.ctypes.data_as(C.c_void_p), sites_out.shape[0], C.byref(k), C.byref(psnr))
        return sites_out[: k.value], float(psnr.value)


def fit(image: np.ndarray, **overrides):
    """Fit one image with the training_config.json schedule; returns (sites, psnr)."""
    h, w = image.shape[:2]
    with Trainer(w, h, **overrides) as tr:
        return tr.fit_host(image)
