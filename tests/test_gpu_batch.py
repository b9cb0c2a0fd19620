"""The lockstep batch of fits (sad_batch_*): every stage of an iteration is one launch over
all images, yet each image's arithmetic is that of a single fit, so every image's sites
must equal, bit for bit, those of its own Trainer fit with the same configuration --
through graph replays and eager launches, with prune events (per-image prune counts from
the bpp rule) and masks.  Integer-exact gradient sums make this a bitwise comparison."""
import numpy as np
import pytest

from sad_gb300.synthetic import synthetic_image

pytestmark = pytest.mark.gpu

SIZES = [(96, 64), (130, 77), (64, 64), (257, 129), (33, 200)]
CFG = dict(iterations=190, n_sites=3000, max_sites=3000, log_freq=0)


def _images():
    return [synthetic_image(w, h, seed=100 + i) for i, (w, h) in enumerate(SIZES)]


def _solo(img, mask=None, **cfg):
    from sad_gb300.trainer import Trainer
    h, w = img.shape[:2]
    with Trainer(w, h, **cfg) as tr:
        tr.set_target(img, mask)
        tr.init()
        tr.run()
        return tr.sites(active_only=False), tr.psnr()


@pytest.mark.parametrize("graphs", [1, 0])
def test_batch_matches_single_fits_bitwise(cuda, graphs):
    from sad_gb300.batch import Batch
    imgs = _images()
    masks = [None] * len(imgs)
    m = np.ones(imgs[1].shape[:2], np.float32)
    m[10:30, 20:60] = 0.0
    masks[1] = m
    with Batch(SIZES, use_graphs=graphs, **CFG) as b:
        for i, img in enumerate(imgs):
            b.set_target(i, img, masks[i])
        b.init()
        b.run(100)  # split runs continue the same fit
        b.run()
        b.synchronize()
        got = [(b.sites(i, active_only=False), b.psnr(i)) for i in range(len(imgs))]
    for i, img in enumerate(imgs):
        want_sites, want_psnr = _solo(img, masks[i], use_graphs=1, **CFG)
        assert got[i][0].shape == want_sites.shape
        np.testing.assert_array_equal(got[i][0].view(np.uint32), want_sites.view(np.uint32), err_msg=f"image {i}")
        assert got[i][1] == want_psnr
        assert (want_sites[:, 0] >= 0).sum() < CFG["n_sites"]  # the prune events ran


def test_batch_of_more_images_than_one_launch_takes(cuda):
    """The per-pixel stages take their images as kernel parameters, up to 96 per launch;
    a larger batch runs each such stage as several launches, with the same results."""
    from sad_gb300.batch import Batch
    rng = np.random.default_rng(7)
    sizes = [(int(rng.integers(16, 49)), int(rng.integers(16, 49))) for _ in range(100)]
    imgs = [synthetic_image(w, h, seed=300 + i) for i, (w, h) in enumerate(sizes)]
    cfg = dict(iterations=60, n_sites=300, max_sites=300, log_freq=0)
    with Batch(sizes, **cfg) as b:
        for i, img in enumerate(imgs):
            b.set_target(i, img)
        b.init()
        b.run()
        b.synchronize()
        got = [b.sites(i, active_only=False) for i in range(len(imgs))]
    for i in (0, 1, 47, 94, 95, 96, 97, 99):
        want, _ = _solo(imgs[i], use_graphs=1, **cfg)
        np.testing.assert_array_equal(got[i].view(np.uint32), want.view(np.uint32), err_msg=f"image {i}")


def test_batch_timing_and_launch_count(cuda):
    from sad_gb300 import _lib
    from sad_gb300.batch import Batch
    lib = _lib.load()
    imgs = _images()[:3]
    with Batch(SIZES[:3], **CFG) as b:
        for i, img in enumerate(imgs):
            b.set_target(i, img)
        b.init()
        b.enable_timing(True)
        k0 = lib.sad_launch_count()
        b.run(40)
        b.synchronize()
        launches = lib.sad_launch_count() - k0
        assert b.gradient_ms() > 0.0
    # one launch per stage for all images: far fewer than per-image launches would take
    assert launches < 40 * 12


def test_batch_rejects_unsupported_schedules(cuda):
    from sad_gb300 import _lib
    from sad_gb300.batch import Batch
    lib = _lib.load()
    img = _images()[0]
    for bad in (dict(n_sites=2000, max_sites=3000), dict(cand_update_passes=2), dict(ssim_weight=0.1)):
        cfg = dict(CFG)
        cfg.update(bad)
        with Batch(SIZES[:1], **cfg) as b:
            b.set_target(0, img)
            st = lib.sad_batch_init(b._h)
            assert st == 4, (bad, lib.sad_last_error())  # SAD_ERR_UNSUPPORTED
