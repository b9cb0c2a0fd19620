"""CPU checks of the oracle: known answers, the reference's own sort and schedule cases,
invariants of the candidate search, and an FP64 finite-difference check of the adjoint."""
import math

import numpy as np
import pytest

import cases


def test_f16_round_to_nearest_even_matches_ieee(orc):
    rng = np.random.default_rng(0)
    vals = np.concatenate([
        np.array([0.0, -0.0, 1.0, -1.0, 65504.0, 65519.99, 65520.0, 1e9, 6.0e-8, 5.960464e-8,
                  2.9802322e-8, 2.9802326e-8, 6.1e-5, 6.097e-5, 1 / 3, 0.1, np.inf, -np.inf],
                 dtype=np.float32),
        rng.normal(0, 100, 2000).astype(np.float32),
        rng.uniform(-1e-4, 1e-4, 2000).astype(np.float32),
    ])
    with np.errstate(over="ignore"):
        want = vals.astype(np.float16).view(np.uint16)
    got = np.array([orc.f32_to_f16_bits(v) for v in vals], dtype=np.uint16)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("w,h", [(1024, 1024), (1000, 600), (256, 256), (1, 1), (3, 2), (4096, 17)])
def test_jump_schedule(orc, w, h):
    # backends/cuda/src/sad_cuda.cu:1157-1183: pow2 >> (min(i, stages - 1) + 1), at least 1
    pow2 = 1
    while pow2 < max(w, h):
        pow2 <<= 1
    stages = int(math.log2(pow2)) if pow2 > 1 else 0
    for i in range(0, 40):
        want = 1 if pow2 <= 1 else max(pow2 >> (min(i, stages - 1) + 1), 1)
        assert orc.jump_step_for_index(i, w, h) == want
        assert orc.pack_jump_step(i, w, h) == ((min(want, 0xFFFF) << 16) | (i & 0xFFFF))
    assert orc.pack_jump_step(70000, w, h) & 0xFFFF == 70000 & 0xFFFF


@pytest.mark.parametrize("bits", [1, 2, 3, 5])
def test_hilbert_index_is_a_continuous_bijection(orc, bits):
    n = 1 << bits
    pos = {}
    for y in range(n):
        for x in range(n):
            pos[orc.hilbert_index(x, y, bits)] = (x, y)
    assert sorted(pos) == list(range(n * n))
    for d in range(n * n - 1):
        (x0, y0), (x1, y1) = pos[d], pos[d + 1]
        assert abs(x0 - x1) + abs(y0 - y1) == 1


def test_hilbert_bits(orc):
    assert orc.hilbert_bits_for_size(1, 1) == 1
    assert orc.hilbert_bits_for_size(1024, 1024) == 10
    assert orc.hilbert_bits_for_size(1025, 3) == 11


@pytest.mark.parametrize("case", cases.sort_cases(), ids=lambda c: c[0])
def test_radix_sort_matches_stable_sort(orc, case):
    name, pairs, max_key, count = case
    got = orc.radix_sort_pairs(pairs, max_key)
    want = cases.expected_sort(pairs, max_key)
    np.testing.assert_array_equal(got, want)
    if max_key > 65536 or pairs[:count, 0].max(initial=0) < 65536:
        # fully sorted by key and stable on the first `count` entries (test_sort.swift:80-111)
        k, v = got[:count, 0].astype(np.int64), got[:count, 1].astype(np.int64)
        assert np.all(np.diff(k) >= 0)
        same = np.diff(k) == 0
        assert np.all(np.diff(v)[same] > 0)


def test_bpp_rule_reference_numbers(orc):
    # 1024^2 at 1.0 bpp from 128,000 sites: target round(1.0 * 1024^2 / 128) = 8192
    out = orc.solve_target_bpp(1.0, 1024, 1024, 128000, 128000, 4000, 1, 20, 3000, 20, 0.01, 1,
                               100, 3000, 40, 0.033, 65536)
    assert int(out[2]) == 8192
    assert abs(out[3] - 1.0) < 1e-6
    assert abs(out[1] - 0.0374797) < 1e-5
    assert abs(out[0] - 0.0113575) < 1e-5
    # prune events at 100, 140, ..., 2980 (73 of them) with the solved percentile
    assert orc.simulate_final_sites(128000, 128000, 4000, 1, 20, 3000, 20, float(out[0]), 1, 100, 3000,
                                    40, float(out[1]), 65536) == 8192


def test_render_single_site_is_flat(orc):
    w = h = 16
    s = np.zeros((1, 10), np.float32)
    s[0] = [5.25, 7.25, 1.0, 2.0, 0.2, 0.4, 0.6, 1.0, 0.0, 0.3]
    c0 = np.full((w * h, 4), 0xFFFFFFFF, np.uint32)
    c1 = c0.copy()
    c0[:, 0] = 0
    out = orc.render(c0, c1, s, w, h)
    np.testing.assert_allclose(out, np.broadcast_to([0.2, 0.4, 0.6], out.shape), atol=1e-6)


def test_render_two_sites_softmax(orc):
    w = h = 8
    s = np.zeros((2, 10), np.float32)
    s[0] = [1.25, 1.25, 2.0, 1.0, 1, 0, 0, 1, 0, 0]
    s[1] = [6.25, 6.25, 1.5, 1.0, 0, 0, 1, 0, 1, 0.5]
    c0 = np.full((w * h, 4), 0xFFFFFFFF, np.uint32)
    c1 = c0.copy()
    c0[:, 0], c0[:, 1] = 0, 1
    out = orc.render(c0, c1, s, w, h)
    inv_s2 = 1.0 / 64.0
    for y in range(h):
        for x in range(w):
            lg = []
            for si in s:
                dx, dy = x - si[0], y - si[1]
                proj = si[7] * dx + si[8] * dy
                perp2 = max(dx * dx + dy * dy - proj * proj, 0.0)
                l1 = math.exp(si[9])
                d2 = max((l1 * proj * proj + perp2 / l1) * inv_s2, 1e-8)
                lg.append(-math.exp(si[2]) * (math.sqrt(d2) - si[3] * math.sqrt(inv_s2)))
            m = max(lg)
            e = [math.exp(v - m) for v in lg]
            wgt = [v / sum(e) for v in e]
            want = wgt[0] * s[0, 4:7] + wgt[1] * s[1, 4:7]
            np.testing.assert_allclose(out[y, x], want, atol=2e-6)


def test_render_all_invalid_is_black_and_ignores_out_of_range(orc):
    w, h, n = 8, 4, 3
    s = np.zeros((n, 10), np.float32)
    s[:, 0] = -1.0  # all inactive
    c0 = np.zeros((w * h, 4), np.uint32)
    c1 = np.full((w * h, 4), n + 5, np.uint32)
    assert np.all(orc.render(c0, c1, s, w, h) == 0.0)


def fd_gradcheck(loss, sites, grad, rows, h=1e-6, rtol=1e-4, floor=1e-3):
    """Central differences (step h) against the adjoint on every parameter of the given
    rows.  The direction enters the metric through max(|d|^2 - (dir.d)^2, 0), which has a
    kink wherever a pixel lies on the site's axis and dir leaves the unit circle, so the
    direction is checked along the unit circle (a rotation by h), the only component the
    optimiser uses (its Adam step is projected on the tangent).  Returns the worst error
    relative to max(|fd|, |grad|, floor)."""
    def fd(i, delta):
        sp, sm = sites.copy(), sites.copy()
        sp[i] += delta
        sm[i] -= delta
        return (loss(sp) - loss(sm)) / 2.0
    worst = 0.0
    for i in rows:
        for c in (0, 1, 2, 3, 4, 5, 6, 9):
            d = np.zeros(10)
            d[c] = h
            f = fd(i, d) / h
            worst = max(worst, abs(f - grad[i, c]) / max(abs(f), abs(grad[i, c]), floor))
        dx, dy = sites[i, 7], sites[i, 8]
        ang = np.arctan2(dy, dx)
        sp, sm = sites.copy(), sites.copy()
        sp[i, 7], sp[i, 8] = np.cos(ang + h), np.sin(ang + h)
        sm[i, 7], sm[i, 8] = np.cos(ang - h), np.sin(ang - h)
        f = (loss(sp) - loss(sm)) / (2 * h)
        a = -dy * grad[i, 7] + dx * grad[i, 8]
        worst = max(worst, abs(f - a) / max(abs(f), abs(a), floor))
    return worst


def test_fp64_gradcheck_of_adjoint(orc):
    """Central differences (h = 1e-6) of the FP64 forward against the FP64 adjoint on all
    per-site parameters of sampled sites, candidate lists held fixed (64x64, 256 sites)."""
    w = h = 64
    img, sites = cases.scene(w, h, 256, seed=3)
    sites = sites.astype(np.float64)
    sites[:, 2] = 3.0  # softer than the training default so every candidate carries weight
    c0, c1 = cases.knn_field(sites.astype(np.float32), w, h)
    inv_s2 = 1.0 / (w * w)
    rng = np.random.default_rng(1)
    gout = rng.normal(size=(h, w, 3))
    loss = lambda s: float(np.sum(orc.render_d(c0, c1, s, w, h, inv_s2) * gout))
    grad = orc.render_backward_d(c0, c1, sites, gout, w, h, inv_s2)
    worst = fd_gradcheck(loss, sites, grad, rng.choice(256, 32, replace=False))
    assert worst < 1e-4, worst


def test_f32_adjoint_tracks_f64(orc):
    w = h = 48
    img, sites = cases.scene(w, h, 180, seed=5)
    c0, c1 = cases.knn_field(sites, w, h)
    inv_s2 = 1.0 / (w * w)
    gout = np.random.default_rng(2).normal(size=(h, w, 3)).astype(np.float32)
    g32, a32 = orc.render_backward(c0, c1, sites, gout, w, h)
    g64 = orc.render_backward_d(c0, c1, sites.astype(np.float64), gout.astype(np.float64), w, h, inv_s2)
    # gradient tolerance: 1e-3 of the summed |per-pixel term| of each component
    assert np.all(np.abs(g32 - g64) <= 1e-3 * a32 + 1e-6)


def _dist(orc, packed, ids, x, y, inv_s2):
    return [orc.packed_distance(packed[i], x, y, inv_s2) if i != 0xFFFFFFFF else np.inf for i in ids]


def test_vpt_lists_sorted_unique_and_monotone(orc):
    w, h, n = 40, 24, 300
    img, sites = cases.scene(w, h, n, seed=7)
    sites[::17, 0] = -1.0  # some inactive
    c0, c1 = cases.random_field(w, h, n, seed=8)
    packed = orc.pack_sites(sites)
    inv_s2 = 1.0 / (w * w)
    o0, o1 = orc.vpt_pass(c0, c1, packed, n, orc.pack_jump_step(0, w, h), 0, w, h, inject=4)
    for p in range(0, w * h, 7):
        x, y = p % w, p // w
        ids = list(o0[p]) + list(o1[p])
        valid = [i for i in ids if i != 0xFFFFFFFF]
        assert len(valid) == len(set(valid))
        assert all(i < n and sites[i, 0] >= 0 for i in valid)
        d = _dist(orc, packed, ids, x, y, inv_s2)
        assert all(d[k] <= d[k + 1] for k in range(7))
        old = [i for i in list(c0[p]) + list(c1[p]) if i < n]
        dold = min(_dist(orc, packed, old, x, y, inv_s2), default=np.inf)
        assert d[0] <= dold


def test_jfa_then_vpt_recall(orc):
    """Candidate quality (the metric of backends/metal/tests/test_jump_schedule.swift:89-136):
    after JFA + VPT passes, the brute-force nearest site is in the top-8 for nearly all
    pixels."""
    w = h = 64
    n = 400
    img, sites = cases.scene(w, h, n, seed=11)
    inv_s2 = 1.0 / (w * w)
    c0 = np.full((w * h, 4), 0xFFFFFFFF, np.uint32)
    c1 = c0.copy()
    c0 = orc.jfa_seed(c0, sites, w, h)
    step = 32
    a, b = c0, c1
    while step >= 1:
        a, b = orc.jfa_flood(a, sites, step, w, h), a
        step //= 2
    c0, c1 = a, b
    packed = orc.pack_sites(sites)
    for i in range(8):
        c0, c1 = orc.vpt_pass(c0, c1, packed, n, orc.pack_jump_step(i, w, h), 0, w, h, inject=4)
    hit = 0
    for p in range(w * h):
        x, y = p % w, p // w
        d = [orc.packed_distance(packed[i], x, y, inv_s2) for i in range(n)]
        best = int(np.argmin(d))
        hit += best in set(c0[p]) | set(c1[p])
    assert hit / (w * h) > 0.98


@pytest.mark.parametrize("w,h,n", [(96, 96, 1000), (128, 80, 3000)])
def test_render_candidate_build_recall(orc, w, h, n):
    """Candidate quality of the render-from-sites build (seed, JFA flood, 16 VPT passes
    with random injection and Hilbert probes) against a brute-force top-8 over all sites,
    by the metrics backends/metal/tests/test_jump_schedule.swift:89-136 prints (Recall@8,
    full-list match), asserted here.  The GPU build returns the same lists
    (test_gpu_trainer.py compares the rendered images)."""
    from checks import packed_dist_np
    _, sites = cases.scene(w, h, n, 21)
    _, (c0, c1) = cases.oracle_render_from_sites(orc, sites, w, h)
    ids = np.concatenate([c0, c1], 1).astype(np.int64)
    inv = 1.0 / max(w, h) ** 2
    ys, xs = np.divmod(np.arange(w * h), w)
    every = np.arange(n)[None, :]
    hits, full, nearest = 0, 0, 0
    for a in range(0, w * h, 512):
        b = min(a + 512, w * h)
        d = packed_dist_np(sites, every, xs[a:b, None].astype(np.float64), ys[a:b, None].astype(np.float64), inv)
        top = np.argsort(d, axis=1, kind="stable")[:, :8]
        for k, p in enumerate(range(a, b)):
            got = set(ids[p])
            hit = len(set(top[k]) & got)
            hits += hit
            full += hit == 8
            nearest += int(top[k, 0]) in got
    npx = w * h
    assert hits / (8 * npx) >= 0.999
    assert full / npx >= 0.99
    assert nearest / npx >= 0.999


def test_init_gradient_weighted_accepts_textured_pixels(orc):
    w, h = 96, 64
    img, _ = cases.scene(w, h, 1, seed=2)
    s = orc.init_gradient_weighted(img, 500)
    act = s[:, 0] >= 0
    assert act.sum() > 400
    assert np.all(s[act, 0] <= w - 1) and np.all(s[act, 1] <= h - 1)
    assert np.all(s[act, 2] > 5.0)  # init_log_tau + 2 grad^0.25 with grad > 0.01
    np.testing.assert_array_equal(s, orc.init_gradient_weighted(img, 500))


def test_tau_diffuse_fixed_point(orc):
    w = h = 16
    n = 50
    img, sites = cases.scene(w, h, n, seed=4)
    c0, c1 = cases.knn_field(sites, w, h)
    g = np.random.default_rng(0).normal(size=n).astype(np.float32)
    # lambda <= 0 copies
    np.testing.assert_array_equal(orc.tau_diffuse(c0, c1, sites, g, g, 0.0, w, h), g)
    # Jacobi converges to (I + lambda L) x = g
    x = g.copy()
    for _ in range(200):
        x = orc.tau_diffuse(c0, c1, sites, g, x, 0.05, w, h)
    x2 = orc.tau_diffuse(c0, c1, sites, g, x, 0.05, w, h)
    np.testing.assert_allclose(x2, x, atol=1e-6)


def test_adam_skips_inactive_and_clamps(orc):
    n = 8
    rng = np.random.default_rng(0)
    s = np.zeros((n, 10), np.float32)
    s[:, 0:2] = 5.0
    s[:, 3] = 1.0
    s[:, 4:7] = 0.999
    s[:, 7] = 1.0
    s[0, 0] = -1.0
    g = rng.normal(size=(10, n)).astype(np.float32) * 1000
    g[4:7] = -1e6
    s2, a2 = orc.adam_update(s, np.zeros((n, 20), np.float32), g, [0.5] * 6, 0.9, 0.999, 1e-8, 1, 16, 16)
    np.testing.assert_array_equal(s2[0], s[0])
    assert np.all(s2[1:, 4:7] <= 1.0) and np.all(s2[1:, 3] >= 1.0)
    assert np.all(np.abs(s2[1:, 9]) <= 4.0)
    np.testing.assert_allclose(np.hypot(s2[1:, 7], s2[1:, 8]), 1.0, atol=1e-6)


def test_prune_pairs_select_smallest_delta(orc):
    n = 100
    s = np.zeros((n, 10), np.float32)
    s[:, 0] = 1.0
    s[::10, 0] = -1.0
    rem = np.random.default_rng(3).normal(size=n).astype(np.float32)
    pairs = orc.prune_pairs(s, rem, 128, 0.5)
    srt = orc.radix_sort_pairs(pairs, 0xFFFFFFFF)
    active = [i for i in range(n) if s[i, 0] >= 0]
    keys = {i: np.float32(max(rem[i] * np.float32(0.5), 0.0)) for i in active}
    want = sorted(active, key=lambda i: (keys[i], i))
    assert list(srt[: len(active), 1]) == want
    assert np.all(srt[len(active):] == 0xFFFFFFFF)


def test_synthetic_generator_is_seeded():
    import sad_gb300.synthetic as syn
    a = syn.synthetic_image(64, 48, seed=5)
    b = syn.synthetic_image(64, 48, seed=5)
    assert a.shape == (48, 64, 3) and a.dtype == np.float32
    np.testing.assert_array_equal(a, b)
    assert a.min() >= 0.0 and a.max() <= 1.0
    s = syn.synthetic_sites(a, 100, seed=5)
    assert s.shape == (100, 10)
    assert np.all((s[:, 0] % 1.0) == 0.25)


def test_sites_txt_round_trip(tmp_path):
    from sad_gb300 import sites_io
    img, s = cases.scene(32, 16, 20, seed=1)
    p = tmp_path / "x_sites.txt"
    sites_io.save_sites(str(p), s, 32, 16)
    back, w, h = sites_io.load_sites(str(p))
    assert (w, h) == (32, 16)
    np.testing.assert_array_equal(back, s)
    with open(p, "a") as f:
        f.write("1 2 0.1 0.2 0.3 4.5 3.0\n")  # 7 columns: dir (1,0), log_aniso 0
        f.write("garbage line\n")
    back, _, _ = sites_io.load_sites(str(p))
    assert back.shape[0] == 21
    np.testing.assert_array_equal(back[-1], np.float32([1, 2, 4.5, 3.0, 0.1, 0.2, 0.3, 1, 0, 0]))
