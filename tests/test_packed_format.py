"""The 16-byte quantised inference sites (the Metal backend's serving format,
backends/metal/sources/utils/packed_inference.swift:86-199, decode
backends/metal/shaders/sad_common.metal:71-120, render packed_render_encoder.metal:3-31).

The reference's packer is Swift and does not run here.  Its decoder is a Metal function
that compiles as plain C++ under a shim of the Metal types: tests/golden/packed_decode.npz
holds the words of the oracle's packer (oracle/sad_oracle.c) decoded by the reference's own
decodePackedSite (tests/golden/make_packed_fixture.py), and the reference's packed render
(computePackedWeights) of one small image.  So the decode and the render are pinned to the
reference, the packer to the reference's decoder by round-trip bounds, and both also by
known-answer words worked out by hand from the format.  The CUDA kernels are
compared with the oracle and the fixture: every word bit-exact except the direction angle,
which may differ by one step where atan2f's last bit differs; the decode is exact except
cos/sin of the angle."""
import ctypes as C

import numpy as np
import pytest

import orc

W, H = 300, 200


def random_sites(n, w, h, seed, inactive_every=17):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 10), np.float32)
    s[:, 0] = rng.uniform(0, w - 1, n)
    s[:, 1] = rng.uniform(0, h - 1, n)
    s[:, 2] = rng.normal(5, 1, n)
    s[:, 3] = rng.uniform(0, 8, n)
    s[:, 4:7] = rng.uniform(-0.1, 1.1, (n, 3))
    th = rng.uniform(0, 2 * np.pi, n)
    r = rng.uniform(0.5, 2.0, n)  # unnormalised directions exercise normalizedDir
    s[:, 7] = np.cos(th) * r
    s[:, 8] = np.sin(th) * r
    s[:, 9] = rng.uniform(-4, 4, n)
    if inactive_every:
        s[::inactive_every, 0:2] = -1.0
    return s


# ---------------------------------------------------------------------------
# oracle, CPU
# ---------------------------------------------------------------------------
def test_known_answer_words():
    # site 0: at the origin, every value at its range minimum, direction +x, log_aniso 0
    # site 1: at (W-1, H-1), every value at its maximum, direction -x, log_aniso 1
    # site 2: inactive, values outside the ranges (they must not widen them)
    s = np.zeros((3, 10), np.float32)
    s[0] = [0, 0, 2.0, 1.0, 0.1, 0.2, 0.3, 1, 0, 0]
    s[1] = [W - 1, H - 1, 6.0, 9.0, 0.9, 0.8, 0.7, -1, 0, 1.0]
    s[2] = [-1, -1, 100, 100, 5, 5, 5, 0, 1, 0]
    packed, quant = orc.pack_inference_sites(s, W, H)
    np.testing.assert_array_equal(quant, np.float32([2.0, 4.0, 1.0, 8.0, 0.1, np.float32(0.9) - np.float32(0.1),
                                                     0.2, np.float32(0.8) - np.float32(0.2), 0.3,
                                                     np.float32(0.7) - np.float32(0.3)]))
    # angle(+x) = 0 -> (0 + pi) / 2pi = 0.5 -> uint(0.5 * 65535 + 0.5) = 32768
    assert packed[0].tolist() == [0, 0, 0, 32768]
    # 15-bit x and y at 32767, 11/11/10-bit colours and 16-bit log_tau/radius at full scale,
    # angle(-x) = pi -> 65535, f16(1.0) = 0x3C00
    assert packed[1].tolist() == [0x3FFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0x3C00FFFF]
    # inactive: clamped position 0, flag bit 30; values clamp to the range ends; dir +y -> 49151
    assert packed[2][0] == 1 << 30
    assert packed[2][1] == 0xFFFFFFFF and packed[2][2] == 0xFFFFFFFF
    assert packed[2][3] == int(0.75 * 65535 + 0.5)
    u = orc.unpack_inference_sites(packed, quant, W, H)
    assert u[2, 0] == -1.0 and u[2, 1] == -1.0
    np.testing.assert_array_equal(u[1, :2], [W - 1, H - 1])
    np.testing.assert_allclose(u[0, :7], [0, 0, 2.0, 1.0, 0.1, 0.2, 0.3], atol=1e-6)
    np.testing.assert_allclose(u[1, :7], [W - 1, H - 1, 6.0, 9.0, 0.9, 0.8, 0.7], atol=1e-6)
    # directions come back within one angle step (2 pi / 65535)
    np.testing.assert_allclose(u[0, 7:], [1, 0, 0], atol=1e-4)
    np.testing.assert_allclose(u[1, 7:], [-1, 0, 1.0], atol=1e-4)


def test_round_trip_bounds():
    s = random_sites(4000, W, H, seed=3)
    packed, quant = orc.pack_inference_sites(s, W, H)
    u = orc.unpack_inference_sites(packed, quant, W, H)
    act = (s[:, 0] >= 0) & (s[:, 1] >= 0)
    a = s[act]
    np.testing.assert_allclose(quant[0::2], [a[:, 2].min(), a[:, 3].min(), a[:, 4].min(), a[:, 5].min(),
                                             a[:, 6].min()])
    err = np.abs(u[act] - a)
    step = lambda scale, levels: scale / levels / 2 + 1e-6 * max(1.0, scale)  # noqa: E731
    assert err[:, 0].max() <= step(W - 1, 32767)
    assert err[:, 1].max() <= step(H - 1, 32767)
    assert err[:, 2].max() <= step(quant[1], 65535)
    assert err[:, 3].max() <= step(quant[3], 65535)
    assert err[:, 4].max() <= step(quant[5], 2047)
    assert err[:, 5].max() <= step(quant[7], 2047)
    assert err[:, 6].max() <= step(quant[9], 1023)
    ang = np.arctan2(a[:, 8], a[:, 7])
    dang = np.angle(np.exp(1j * (np.arctan2(u[act, 8], u[act, 7]) - ang)))
    assert np.abs(dang).max() <= np.pi / 65535 + 1e-5
    np.testing.assert_array_equal(u[act, 9], a[:, 9].astype(np.float16).astype(np.float32))
    assert np.all(u[~act, :2] == -1.0)
    assert np.all((packed[~act, 0] >> 30) & 1) and not np.any((packed[act, 0] >> 30) & 1)


def _fixture_cases():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "packed_decode.npz"))
    for c in ("a", "b", "edges", "one"):
        w, h = (int(v) for v in z[f"{c}_size"])
        yield (c, z[f"{c}_sites"], z[f"{c}_words"], z[f"{c}_quant"], w, h, z[f"{c}_decoded"],
               z[f"{c}_active"].astype(bool))


EXACT = [0, 1, 2, 3, 4, 5, 6, 9]  # every decoded field but the direction (cos/sin of the angle)


def test_oracle_decode_matches_reference_decoder():
    """The oracle's unpack against the reference's decodePackedSite on the same words:
    bit-exact (the direction within 2 ulps, for another host's libm); inactive sites by the
    decoder's flag."""
    for c, sites, words, quant, w, h, ref, act in _fixture_cases():
        np.testing.assert_array_equal(words, orc.pack_inference_sites(sites, w, h)[0])  # packer unchanged
        u = orc.unpack_inference_sites(words, quant, w, h)
        np.testing.assert_array_equal(u[act][:, EXACT].view(np.uint32), ref[act][:, EXACT].view(np.uint32), err_msg=c)
        ulp = np.abs(u[act][:, 7:9].view(np.int32).astype(np.int64) - ref[act][:, 7:9].view(np.int32).astype(np.int64))
        assert ulp.size == 0 or ulp.max() <= 2, c
        assert np.all(u[~act, :2] == -1.0), c


def test_packer_round_trip_through_reference_decoder():
    """The oracle packer's words, decoded by the reference's decoder, give back every active
    site within half a quantisation step per field (an angle step for the direction, f16
    for log_aniso), and the decoder reads inactive sites as inactive."""
    for c, sites, words, quant, w, h, ref, act in _fixture_cases():
        want_act = (sites[:, 0] >= 0) & (sites[:, 1] >= 0)
        np.testing.assert_array_equal(act, want_act, err_msg=c)
        a, u = sites[act], ref[act]
        if not len(a):
            continue
        step = lambda scale, levels: scale / levels / 2 + 1e-6 * max(1.0, scale)  # noqa: E731
        err = np.abs(u - a)
        assert err[:, 0].max() <= step(w - 1, 32767) and err[:, 1].max() <= step(h - 1, 32767), c
        for k, (qs, levels) in enumerate([(quant[1], 65535), (quant[3], 65535), (quant[5], 2047),
                                          (quant[7], 2047), (quant[9], 1023)]):
            assert err[:, 2 + k].max() <= step(qs, levels), (c, k)
        ang = np.arctan2(a[:, 8], a[:, 7])
        dang = np.angle(np.exp(1j * (np.arctan2(u[:, 8], u[:, 7]) - ang)))
        assert np.abs(dang).max() <= np.pi / 65535 + 1e-5, c
        np.testing.assert_array_equal(u[:, 9], a[:, 9].astype(np.float16).astype(np.float32), err_msg=c)


def _render_case():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "packed_decode.npz"))
    w, h = (int(v) for v in z["render_size"])
    return (z["render_words"], z["render_quant"], z["render_c0"], z["render_c1"], float(z["render_inv_s2"][0]),
            w, h, z["render_rgb"])


def test_oracle_render_matches_reference_packed_render():
    """The oracle's render of its decoded sites against the reference's packed render
    (computePackedWeights of renderVoronoiPacked) of the same words and candidate field:
    equal here; 1e-6 allows another host's libm."""
    words, quant, c0, c1, inv_s2, w, h, want = _render_case()
    dec = orc.unpack_inference_sites(words, quant, w, h)
    got = orc.render(c0, c1, dec, w, h, inv_s2=inv_s2)
    assert np.max(np.abs(got - want)) <= 1e-6


def test_degenerate_sets():
    s = random_sites(10, W, H, seed=1, inactive_every=1)  # all inactive
    packed, quant = orc.pack_inference_sites(s, W, H)
    np.testing.assert_array_equal(quant, np.float32([0, 1e-6] * 5))
    assert np.all(packed[:, 0] == 1 << 30)
    s = random_sites(5, W, H, seed=2, inactive_every=0)
    s[1, 2] = np.inf
    s[2, 3] = np.nan
    s[3, 9] = np.nan
    packed, quant = orc.pack_inference_sites(s, W, H)
    assert packed[1, 2] & 0xFFFF == 0          # non-finite log_tau packs as the range minimum
    assert packed[2, 2] >> 16 == 0             # non-finite radius likewise
    assert packed[3, 3] >> 16 == 0             # non-finite log_aniso packs as 0
    assert np.isfinite(quant).all()
    one = orc.pack_inference_sites(s[:1], 1, 1)[0]  # 1x1 image: positions pack to 0
    assert one[0, 0] == 0


# ---------------------------------------------------------------------------
# CUDA kernels against the oracle
# ---------------------------------------------------------------------------
def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _gpu_pack(lib, sites, w, h):
    import torch
    n = sites.shape[0]
    packed = torch.zeros((max(n, 1), 4), dtype=torch.int32, device="cuda")
    quant = torch.zeros(10, dtype=torch.float32, device="cuda")
    d = torch.from_numpy(sites).cuda() if n else torch.zeros((1, 10), device="cuda")
    assert lib.sad_pack_inference_sites(_ptr(d), n, w, h, _ptr(packed), _ptr(quant), None) == 0, \
        lib.sad_last_error()
    torch.cuda.synchronize()
    return packed[:n].cpu().numpy().view(np.uint32), quant.cpu().numpy()


def _gpu_unpack(lib, packed, quant, w, h):
    import torch
    p = torch.from_numpy(packed.view(np.int32)).cuda()
    q = torch.from_numpy(quant).cuda()
    out = torch.zeros((packed.shape[0], 10), dtype=torch.float32, device="cuda")
    assert lib.sad_unpack_inference_sites(_ptr(p), _ptr(q), packed.shape[0], w, h, _ptr(out), None) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _assert_words_match(got, want):
    np.testing.assert_array_equal(got[:, :3], want[:, :3])
    np.testing.assert_array_equal(got[:, 3] >> 16, want[:, 3] >> 16)
    d = got[:, 3].astype(np.int64) & 0xFFFF
    e = want[:, 3].astype(np.int64) & 0xFFFF
    assert np.abs(d - e).max() <= 1
    assert np.mean(d == e) > 0.999


@pytest.mark.gpu
@pytest.mark.parametrize("n,w,h", [(5000, W, H), (131072, 1024, 1024), (1, 1, 1), (7, 32768, 3)])
def test_gpu_pack_matches_oracle(sadlib, cuda, n, w, h):
    s = random_sites(n, w, h, seed=n)
    got, gq = _gpu_pack(sadlib, s, w, h)
    want, wq = orc.pack_inference_sites(s, w, h)
    np.testing.assert_array_equal(gq, wq)
    _assert_words_match(got, want)
    u = _gpu_unpack(sadlib, want, wq, w, h)
    uo = orc.unpack_inference_sites(want, wq, w, h)
    np.testing.assert_array_equal(u[:, [0, 1, 2, 3, 4, 5, 6, 9]], uo[:, [0, 1, 2, 3, 4, 5, 6, 9]])
    np.testing.assert_allclose(u[:, 7:9], uo[:, 7:9], rtol=0, atol=4e-7)


@pytest.mark.gpu
def test_gpu_unpack_matches_reference_decoder(sadlib, cuda):
    """The CUDA unpack kernel on the fixture's words against the reference's decoder:
    bit-exact except the direction (CUDA cosf/sinf, within 4e-7)."""
    for c, sites, words, quant, w, h, ref, act in _fixture_cases():
        u = _gpu_unpack(sadlib, words, quant, w, h)
        np.testing.assert_array_equal(u[act][:, EXACT].view(np.uint32), ref[act][:, EXACT].view(np.uint32), err_msg=c)
        np.testing.assert_allclose(u[act][:, 7:9], ref[act][:, 7:9], rtol=0, atol=4e-7, err_msg=c)
        assert np.all(u[~act, :2] == -1.0), c
        got, gq = _gpu_pack(sadlib, sites, w, h)
        np.testing.assert_array_equal(gq, quant)
        _assert_words_match(got, words)


@pytest.mark.gpu
def test_gpu_render_packed_matches_reference(sadlib, cuda):
    """The CUDA packed render against the reference's packed render of the same words and
    candidate field (CUDA expf/cosf/sinf: the render tolerance, 1e-4)."""
    import torch
    words, quant, c0, c1, inv_s2, w, h, want = _render_case()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()  # noqa: E731
    dc0, dc1, dp = t(c0), t(c1), t(words)
    dq = torch.from_numpy(quant).cuda()
    out = torch.zeros((h, w, 3), device="cuda")
    assert sadlib.sad_render_packed(_ptr(dc0), _ptr(dc1), _ptr(out), _ptr(dp), _ptr(dq), inv_s2, words.shape[0],
                                    w, h, w, h, None) == 0
    torch.cuda.synchronize()
    assert np.max(np.abs(out.cpu().numpy() - want)) <= 1e-4


@pytest.mark.gpu
def test_gpu_pack_edge_cases(sadlib, cuda):
    s = random_sites(64, W, H, seed=9, inactive_every=1)
    got, gq = _gpu_pack(sadlib, s, W, H)
    want, wq = orc.pack_inference_sites(s, W, H)
    np.testing.assert_array_equal(gq, wq)
    _assert_words_match(got, want)
    s = random_sites(64, W, H, seed=10, inactive_every=0)
    s[3, 2], s[4, 3], s[5, 9], s[6, 4] = np.inf, np.nan, -np.inf, np.nan
    got, gq = _gpu_pack(sadlib, s, W, H)
    want, wq = orc.pack_inference_sites(s, W, H)
    np.testing.assert_array_equal(gq, wq)
    np.testing.assert_array_equal(got[[3, 4, 5], :], want[[3, 4, 5], :])
    _, q0 = _gpu_pack(sadlib, np.zeros((0, 10), np.float32), W, H)
    np.testing.assert_array_equal(q0, np.float32([0, 1e-6] * 5))
    import torch
    big = torch.zeros((1, 10), device="cuda")
    assert sadlib.sad_pack_inference_sites(_ptr(big), 1, 40000, 10, _ptr(big), _ptr(big), None) != 0


@pytest.mark.gpu
def test_gpu_render_packed(sadlib, cuda):
    import torch
    import cases
    w, h = 160, 120
    _, s = cases.scene(w, h, 900, 21)
    s[::13, 0:2] = -1.0
    packed, quant = orc.pack_inference_sites(s, w, h)
    decoded = orc.unpack_inference_sites(packed, quant, w, h)
    c0, c1 = cases.random_field(w, h, s.shape[0], 21)  # empty, out-of-range and repeated ids
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()  # noqa: E731
    dc0, dc1, dp = t(c0), t(c1), t(packed)
    dq = torch.from_numpy(quant).cuda()
    out_p = torch.zeros((h, w, 3), device="cuda")
    out_r = torch.zeros((h, w, 3), device="cuda")
    inv = 1.0 / (max(w, h) ** 2)
    assert sadlib.sad_render_packed(_ptr(dc0), _ptr(dc1), _ptr(out_p), _ptr(dp), _ptr(dq), inv, s.shape[0],
                                    w, h, w, h, None) == 0
    dec_host = _gpu_unpack(sadlib, packed, quant, w, h)
    dec = torch.from_numpy(dec_host).cuda()
    assert sadlib.sad_render(_ptr(dc0), _ptr(dc1), _ptr(out_r), _ptr(dec), inv, s.shape[0], w, h, w, h,
                             None) == 0
    torch.cuda.synchronize()
    # same decode on the device: the packed render equals the render of the decoded sites
    assert torch.equal(out_p, out_r)
    got = out_p.cpu().numpy().reshape(-1)
    # the oracle render of the same decoded sites: the render tolerance of the f32 path
    assert np.max(np.abs(got - orc.render(c0, c1, dec_host, w, h).reshape(-1))) <= 1e-4
    # the oracle's own decode differs only in cos/sin's last bits, which the sharp softmax
    # (tau up to e^7) can amplify at a few pixels
    assert np.max(np.abs(got - orc.render(c0, c1, decoded, w, h).reshape(-1))) <= 5e-3


@pytest.mark.gpu
def test_gpu_render_packed_from_sites(sadlib, cuda):
    import torch
    from sad_gb300 import _lib
    w, h = 192, 160
    s = random_sites(1500, w, h, seed=33, inactive_every=0)
    packed, quant = orc.pack_inference_sites(s, w, h)
    cfg = _lib.RenderConfig()
    sadlib.sad_render_config_default(C.byref(cfg))
    n = s.shape[0]
    dp = torch.from_numpy(packed.view(np.int32)).cuda()
    dq = torch.from_numpy(quant).cuda()
    nb = sadlib.sad_render_packed_scratch_bytes(n, w, h, cfg.cand_downscale)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    out_p = torch.zeros((h, w, 3), device="cuda")
    assert sadlib.sad_render_packed_from_sites(C.byref(cfg), _ptr(dp), _ptr(dq), n, w, h, _ptr(out_p),
                                               _ptr(scratch), nb, None) == 0, sadlib.sad_last_error()
    dec = torch.from_numpy(_gpu_unpack(sadlib, packed, quant, w, h)).cuda()
    nb2 = sadlib.sad_render_scratch_bytes(n, w, h, cfg.cand_downscale)
    scratch2 = torch.empty(nb2, dtype=torch.uint8, device="cuda")
    out_r = torch.zeros((h, w, 3), device="cuda")
    assert sadlib.sad_render_from_sites(C.byref(cfg), _ptr(dec), n, w, h, _ptr(out_r), _ptr(scratch2), nb2,
                                        None) == 0
    torch.cuda.synchronize()
    assert torch.equal(out_p, out_r)
    assert sadlib.sad_render_packed_from_sites(C.byref(cfg), _ptr(dp), _ptr(dq), n, w, h, _ptr(out_p),
                                               _ptr(scratch), nb - 1, None) != 0


@pytest.mark.gpu
def test_gpu_trainer_render_packed(sadlib, cuda):
    import torch
    from sad_gb300 import _lib
    from sad_gb300.synthetic import synthetic_image
    w, h = 128, 96
    img = synthetic_image(w, h, seed=4)
    cfg = _lib.TrainConfig()
    sadlib.sad_train_config_default(C.byref(cfg))
    cfg.n_sites, cfg.max_sites, cfg.iterations, cfg.log_freq = 800, 800, 150, 0
    t = C.c_void_p()
    assert sadlib.sad_trainer_create(C.byref(cfg), w, h, C.byref(t)) == 0
    try:
        tgt = np.ascontiguousarray(img, np.float32)
        assert sadlib.sad_trainer_set_target_host(t, tgt.ctypes.data_as(C.c_void_p), None) == 0
        assert sadlib.sad_trainer_init(t, None, 0) == 0
        assert sadlib.sad_trainer_run(t, cfg.iterations) == 0
        p_full, p_packed = C.c_float(), C.c_float()
        rgb = torch.zeros((h, w, 3), device="cuda")
        assert sadlib.sad_trainer_render(t, None, C.byref(p_full)) == 0
        q = (C.c_float * 10)()
        assert sadlib.sad_trainer_render_packed(t, _ptr(rgb), C.byref(p_packed), q) == 0, sadlib.sad_last_error()
        info = _lib.TrainerInfo()
        sadlib.sad_trainer_info(t, C.byref(info))
        sites = np.zeros((info.site_buffer, 10), np.float32)
        k = C.c_int()
        assert sadlib.sad_trainer_get_sites(t, sites.ctypes.data_as(C.c_void_p), info.site_buffer, 0,
                                            C.byref(k)) == 0
        _, wq = orc.pack_inference_sites(sites[:k.value], w, h)
        np.testing.assert_array_equal(np.frombuffer(q, np.float32), wq)
        # 16-byte sites lose a little accuracy, never most of it
        assert p_full.value - 1.5 < p_packed.value <= p_full.value + 0.05
        assert float(rgb.abs().sum()) > 0
    finally:
        sadlib.sad_trainer_destroy(t)
