"""Concurrent fits and renders (executor.cpp) and trainers in caller-owned memory.

Fits sum their gradients in fixed point and renders have no cross-pixel reductions, so a
request run concurrently with others must give bitwise the result of the same request run
alone: sad_trainer_fit_host on its own handle, or sad_render_from_sites."""
import ctypes as C

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


def small_cfg(**kw):
    from sad_gb300.config import train_config
    base = dict(n_sites=600, max_sites=600, iterations=80, target_bpp=0.0, prune_percentile=0.02,
                prune_start=20, prune_freq=10, prune_end=60, log_freq=0, cand_hilbert_window=16)
    base.update(kw)
    return train_config(**base)


def solo_fit(img, cfg):
    from sad_gb300.trainer import Trainer
    h, w = img.shape[:2]
    with Trainer(w, h, cfg) as tr:
        return tr.fit_host(img, np.zeros((max(cfg.max_sites, cfg.n_sites, 2 * w * h), 10), np.float32))


def solo_render(sites, w, h):
    from sad_gb300 import _lib
    lib = _lib.load()
    cfg = _lib.RenderConfig()
    lib.sad_render_config_default(C.byref(cfg))
    n = sites.shape[0]
    nb = lib.sad_render_scratch_bytes(n, w, h, cfg.cand_downscale)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    d = torch.from_numpy(np.ascontiguousarray(sites)).cuda()
    out = torch.zeros((h, w, 3), device="cuda")
    assert lib.sad_render_from_sites(C.byref(cfg), C.c_void_p(d.data_ptr()), n, w, h, C.c_void_p(out.data_ptr()),
                                     C.c_void_p(scratch.data_ptr()), nb, None) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_trainer_in_caller_memory(cuda):
    from sad_gb300 import _lib
    lib = _lib.load()
    img = cases.scene(80, 64, 2)[0]
    cfg = small_cfg()
    need = lib.sad_trainer_memory_bytes(C.byref(cfg), 80, 64)
    assert need > 0
    mem = torch.empty(need, dtype=torch.uint8, device="cuda")
    t = C.c_void_p()
    assert lib.sad_trainer_create_in(C.byref(cfg), 80, 64, C.c_void_p(mem.data_ptr()), need - 1, C.byref(t)) != 0
    assert b"sad_trainer_memory_bytes" in lib.sad_last_error()
    assert lib.sad_trainer_create_in(C.byref(cfg), 80, 64, C.c_void_p(mem.data_ptr()), need, C.byref(t)) == 0
    try:
        out = np.zeros((4096, 10), np.float32)
        k, psnr = C.c_int(), C.c_float()
        assert lib.sad_trainer_fit_host(t, img.ctypes.data_as(C.c_void_p), None, out.ctypes.data_as(C.c_void_p),
                                        out.shape[0], C.byref(k), C.byref(psnr)) == 0
    finally:
        lib.sad_trainer_destroy(t)
    want, want_psnr = solo_fit(img, cfg)
    assert psnr.value == want_psnr
    np.testing.assert_array_equal(out[: k.value], want)


@pytest.mark.parametrize("workers,budget", [(4, 0), (3, 1)])
def test_executor_matches_solo_requests(cuda, workers, budget):
    from sad_gb300.executor import Executor
    sizes = [(64, 48), (96, 96), (128, 80), (72, 120), (64, 64), (100, 60)]
    imgs = [cases.scene(w, h, 10 + i)[0] for i, (w, h) in enumerate(sizes)]
    cfgs = [small_cfg(n_sites=300 + 100 * i, max_sites=300 + 100 * i) for i in range(len(sizes))]
    mask = np.ones((48, 64), np.float32)
    mask[:, :20] = 0.0
    scenes = [cases.scene(w, h, 40 + i, ) for i, (w, h) in enumerate([(160, 120), (96, 200), (256, 256)])]
    render_sites = [s for _, s in scenes]
    render_sizes = [(160, 120), (96, 200), (256, 256)]
    with Executor(workers=workers, hbm_budget_bytes=budget) as ex:
        fits = [ex.submit_fit(img, config=cfg) for img, cfg in zip(imgs, cfgs)]
        masked = ex.submit_fit(imgs[0], mask=mask, config=cfgs[0])
        renders = [ex.submit_render(s, w, h) for s, (w, h) in zip(render_sites, render_sizes)]
        ex.wait_all()
        for req in fits + [masked] + renders:
            assert req.res.status == 0, req.res.message
            assert req.run_ms > 0.0 and req.queue_ms >= 0.0
        for req, img, cfg in zip(fits, imgs, cfgs):
            sites, psnr = req.result()
            want, want_psnr = solo_fit(img, cfg)
            assert psnr == want_psnr
            np.testing.assert_array_equal(sites, want)
        for req, s, (w, h) in zip(renders, render_sites, render_sizes):
            np.testing.assert_array_equal(req.result(), solo_render(s, w, h))
        sites_m, psnr_m = masked.result()
        assert psnr_m != fits[0].result()[1]  # the mask changes the fit


def test_executor_argument_errors_and_drain(cuda):
    from sad_gb300 import _lib
    from sad_gb300.executor import Executor
    ex = Executor(workers=2)
    img = cases.scene(64, 64, 7)[0]
    with pytest.raises(RuntimeError):
        ex.submit_fit(img, config=small_cfg(n_sites=0))
    with pytest.raises(RuntimeError):
        ex.submit_render(np.zeros((0, 10), np.float32), 64, 64)
    reqs = [ex.submit_fit(img, config=small_cfg(iterations=30)) for _ in range(3)]
    ex.close()  # runs what is queued, then joins
    out = [r.res for r in reqs]
    assert all(o.status == 0 for o in out)
    assert len({float(o.psnr) for o in out}) == 1
    lib = _lib.load()
    cfg = _lib.ExecutorConfig()
    lib.sad_executor_config_default(C.byref(cfg))
    assert cfg.workers == 8 and cfg.hbm_budget_bytes == 0 and cfg.max_running_fits == 0
    cfg.workers = 0
    h = C.c_void_p()
    assert lib.sad_executor_create(C.byref(cfg), C.byref(h)) != 0


def test_executor_holds_unreferenced_requests(cuda):
    """Requests whose handles the caller drops still own their host buffers until done."""
    import gc
    from sad_gb300.executor import Executor
    img = cases.scene(64, 64, 8)[0]
    ex = Executor(workers=2)
    for _ in range(4):
        ex.submit_fit(img, config=small_cfg(iterations=20))
    ex.submit_render(cases.scene(64, 64, 9)[1], 64, 64)
    gc.collect()
    ex.wait_all()
    kept = ex.submit_fit(img, config=small_cfg(iterations=20))
    gc.collect()
    ex.close()
    assert kept.res.status == 0 and kept.result()[1] > 0


def test_executor_fit_cap_lets_renders_pass(cuda):
    """max_running_fits=1: fits run one at a time (their run intervals do not overlap) while
    renders queued behind a waiting fit still start; results stay those of solo runs."""
    import time
    from sad_gb300.executor import Executor
    imgs = [cases.scene(96, 80, 60 + i)[0] for i in range(3)]
    cfg = small_cfg(iterations=120)
    _, sites = cases.scene(128, 96, 70)
    with Executor(workers=4, max_running_fits=1) as ex:
        t0 = time.perf_counter()
        fits = [ex.submit_fit(img, config=cfg) for img in imgs]
        renders = [ex.submit_render(sites, 128, 96) for _ in range(3)]
        ex.wait_all()
        span = 1e3 * (time.perf_counter() - t0)
        iv = sorted((r.queue_ms, r.queue_ms + r.run_ms) for r in fits)
        for (a0, a1), (b0, b1) in zip(iv, iv[1:]):
            assert b0 >= a1 - 0.5, iv  # submission times differ by well under 0.5 ms
        # the renders did not wait for all three fits
        assert min(r.queue_ms for r in renders) < iv[-1][0]
        assert max(b for _, b in iv) <= span + 1.0
        for req, img in zip(fits, imgs):
            sites_out, psnr = req.result()
            want, want_psnr = solo_fit(img, cfg)
            assert psnr == want_psnr
            np.testing.assert_array_equal(sites_out, want)
        want_r = solo_render(sites, 128, 96)
        for r in renders:
            np.testing.assert_array_equal(r.result(), want_r)



def test_executor_cancel_queued_request(cuda):
    """A request still queued behind a running fit is withdrawn: its result reports the
    cancellation, and the requests around it complete with their solo results."""
    from sad_gb300.executor import Executor, RequestError
    imgs = [cases.scene(96, 80, 80 + i)[0] for i in range(3)]
    cfg = small_cfg(iterations=200)
    with Executor(workers=1) as ex:  # one worker: requests run strictly one after another
        first = ex.submit_fit(imgs[0], config=cfg)
        withdrawn = ex.submit_fit(imgs[1], config=cfg)
        last = ex.submit_fit(imgs[2], config=cfg)
        assert ex.cancel(withdrawn)
        with pytest.raises(RequestError, match="cancelled"):
            withdrawn.result()
        assert withdrawn.res.status == 6  # SAD_ERR_CANCELLED
        ex.wait_all()
        assert not ex.cancel(first)  # finished: nothing to withdraw
        for req, img in ((first, imgs[0]), (last, imgs[2])):
            sites_out, psnr = req.result()
            want, want_psnr = solo_fit(img, cfg)
            assert psnr == want_psnr
            np.testing.assert_array_equal(sites_out, want)


def test_executor_survives_refused_slabs(cuda):
    """Host-side failure injection (no GPU fault): refused slab allocations fail exactly
    their requests with an out-of-memory status and release their budget; the executor
    keeps serving, and the other requests give their solo results."""
    from sad_gb300.executor import Executor, RequestError
    _, sites = cases.scene(96, 64, 90)
    want = solo_render(sites, 96, 64)
    budget = 1 << 30
    with Executor(workers=2, hbm_budget_bytes=budget) as ex:
        ex.inject_slab_failures(2)
        reqs = [ex.submit_render(sites, 96, 64) for _ in range(6)]
        ex.wait_all()
        failed = [r for r in reqs if r.res.status != 0]
        assert len(failed) == 2
        for r in failed:
            assert r.res.status == 3  # SAD_ERR_OUT_OF_MEMORY
            with pytest.raises(RequestError, match="injected"):
                r.result()
        for r in reqs:
            if r.res.status == 0:
                np.testing.assert_array_equal(r.result(), want)
        # the refused requests' budget was released: a full-budget sequence still runs
        more = [ex.submit_render(sites, 96, 64) for _ in range(3)]
        ex.wait_all()
        for r in more:
            np.testing.assert_array_equal(r.result(), want)
