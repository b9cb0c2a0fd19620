"""Degenerate image sizes through the whole fit and the render from sites: one pixel, one
row, one column, odd sizes, more sites than pixels.  The oracle's fit runs the same cases
(tests/test_oracle_cpu.py covers its side); here the device path must stay finite,
reproducible and improving."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = [(1, 1), (2, 2), (1, 64), (64, 1), (3, 2), (17, 5)]


@pytest.mark.parametrize("w,h", SIZES)
def test_fit_at_degenerate_sizes(cuda, w, h):
    from sad_gb300.config import train_config
    from sad_gb300.trainer import Trainer
    img = np.random.default_rng(w * 100 + h).uniform(0, 1, (h, w, 3)).astype(np.float32)
    cfg = train_config(log_freq=0, n_sites=4, max_sites=8, iterations=40, target_bpp=0.0, prune_start=5,
                       prune_freq=5, prune_end=30, cand_hilbert_window=4)
    out = []
    for _ in range(2):
        with Trainer(w, h, cfg) as tr:
            tr.set_target(img)
            tr.init()
            p0 = tr.psnr()
            tr.run()
            p1 = tr.psnr()
            out.append((p0, p1, tr.sites(active_only=False)))
    (p0, p1, s0), (q0, q1, s1) = out
    assert np.isfinite(p0) and np.isfinite(p1) and np.isfinite(s0).all()
    assert p1 >= p0 - 1e-3
    assert (p0, p1) == (q0, q1)
    np.testing.assert_array_equal(s0, s1)


@pytest.mark.parametrize("w,h,n", [(1, 1, 1), (1, 1, 3), (2, 3, 1), (1, 50, 7), (50, 1, 7), (9, 7, 200)])
def test_render_from_sites_at_degenerate_sizes(cuda, w, h, n):
    from sad_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(n)
    s = np.zeros((n, 10), np.float32)
    s[:, 0] = rng.uniform(0, w, n)
    s[:, 1] = rng.uniform(0, h, n)
    s[:, 2], s[:, 3] = 5.0, 4.0
    s[:, 4:7] = rng.uniform(0.2, 0.8, (n, 3))
    s[:, 7] = 1.0
    cfg = _lib.RenderConfig()
    lib.sad_render_config_default(C.byref(cfg))
    nb = lib.sad_render_scratch_bytes(n, w, h, cfg.cand_downscale)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    d = torch.from_numpy(s).cuda()
    out = torch.full((h, w, 3), -1.0, device="cuda")
    assert lib.sad_render_from_sites(C.byref(cfg), C.c_void_p(d.data_ptr()), n, w, h, C.c_void_p(out.data_ptr()),
                                     C.c_void_p(scratch.data_ptr()), nb, None) == 0, lib.sad_last_error()
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    # every pixel is written, and is a convex combination of the site colours
    assert np.isfinite(o).all()
    assert o.min() >= 0.2 - 1e-5 and o.max() <= 0.8 + 1e-5
