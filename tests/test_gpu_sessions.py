"""Resident fit sessions of the executor (sad_executor_open_fit / submit_continue /
close_fit): a fit whose sites, Adam moments, candidate fields and device counters stay on
the device between requests.  A session continued in several requests must give the sites
and PSNR of one uninterrupted fit of the same configuration, bit for bit, also when its
requests interleave with other fits, renders and sessions; its slab counts against the
HBM budget until it is closed."""
import numpy as np
import pytest

import cases
from test_gpu_executor import small_cfg, solo_fit, solo_render

pytestmark = pytest.mark.gpu


def _same(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_session_continued_equals_uninterrupted_fit(cuda):
    from sad_gb300.executor import Executor
    img = cases.scene(96, 72, 2, 7)[0]
    cfg = small_cfg()
    want_sites, want_psnr = solo_fit(img, cfg)
    with Executor(workers=2) as ex:
        s = ex.open_fit(img, config=cfg)
        p0 = s.opened.result()
        parts = [s.continue_fit(k) for k in (25, 30, 100)]  # the last stops at the schedule's end
        got = [p.result() for p in parts]
        s.close().result()
    assert [g[2] for g in got] == [25, 55, 80]
    assert _same(got[-1][0], want_sites)
    assert got[-1][1] == want_psnr
    assert p0 < got[0][1] < got[-1][1]  # the fit improves across requests


def test_sessions_interleave_with_fits_and_renders(cuda):
    from sad_gb300.executor import Executor
    imgs = [cases.scene(96, 72, 2, 11 + i)[0] for i in range(3)]
    cfg = small_cfg()
    want = [solo_fit(im, cfg) for im in imgs]
    rng = np.random.default_rng(3)
    sites = rng.random((500, 10)).astype(np.float32)
    sites[:, 0:2] *= 128
    sites[:, 2], sites[:, 3] = 5.0, 4.0
    sites[:, 7], sites[:, 8] = 1.0, 0.0
    sites[:, 9] = 0.0
    want_render = solo_render(sites, 128, 128)
    with Executor(workers=4) as ex:
        s0 = ex.open_fit(imgs[0], config=cfg)
        s1 = ex.open_fit(imgs[1], config=cfg)
        fit = ex.submit_fit(imgs[2], config=cfg)
        r0 = ex.submit_render(sites, 128, 128)
        a = [s0.continue_fit(40, sites=False), s1.continue_fit(10, sites=False)]
        r1 = ex.submit_render(sites, 128, 128)
        b = [s0.continue_fit(40), s1.continue_fit(70)]
        got0, got1 = b[0].result(), b[1].result()
        s0.close()
        s1.close()
        ex.wait_all()
        assert [x.result()[2] for x in a] == [40, 10]
        assert np.array_equal(r0.result(), want_render) and np.array_equal(r1.result(), want_render)
        assert _same(fit.result()[0], want[2][0])
    assert got0[2] == got1[2] == 80
    assert _same(got0[0], want[0][0]) and got0[1] == want[0][1]
    assert _same(got1[0], want[1][0]) and got1[1] == want[1][1]


def test_session_holds_budget_until_closed(cuda):
    """Under a budget that holds one session's slab, a second session opens only after the
    first is closed (its slab stays charged between requests)."""
    import ctypes as C

    from sad_gb300 import _lib
    from sad_gb300.executor import Executor
    lib = _lib.load()
    img = cases.scene(96, 72, 2, 21)[0]
    cfg = small_cfg()
    need = lib.sad_trainer_memory_bytes(C.byref(cfg), 96, 72)
    with Executor(workers=2, hbm_budget_bytes=int(need * 1.5)) as ex:
        s0 = ex.open_fit(img, config=cfg)
        s0.opened.result()
        s1 = ex.open_fit(img, config=cfg)
        c0 = s0.continue_fit(80)
        got0 = c0.result()
        assert not s1.opened._done and s1.opened.res.run_ms == 0.0  # still waiting for memory
        s0.close().result()
        s1.opened.result()
        got1 = s1.continue_fit(80).result()
        s1.close()
        ex.wait_all()
    assert _same(got0[0], got1[0])


def test_session_errors(cuda):
    import ctypes as C

    from sad_gb300 import _lib
    from sad_gb300.executor import Executor, RequestError
    img = cases.scene(64, 48, 2, 31)[0]
    cfg = small_cfg()
    with Executor(workers=1) as ex:
        res, ticket = _lib.RequestResult(), C.c_uint64(0)
        assert ex._lib.sad_executor_close_fit(ex._h, 12345, C.byref(res), C.byref(ticket)) != 0
        assert b"unknown or closed session" in ex._lib.sad_last_error()
        s = ex.open_fit(img, config=cfg)
        s.close().result()
        with pytest.raises(RuntimeError, match="unknown or closed session"):
            s.continue_fit(10)
        # a session whose slab is refused fails its open; its continue reports that, and
        # its close still succeeds
        ex.inject_slab_failures(1)
        bad = ex.open_fit(img, config=cfg)
        with pytest.raises(RequestError, match="refused"):
            bad.opened.result()
        with pytest.raises(RequestError, match="refused"):
            bad.continue_fit(10).result()
        bad.close().result()
        ex.wait_all()
