"""Parity against the reference's own kernels: golden fixtures in tests/golden/*.npz were
produced by running the reference's CUDA kernels (backends/cuda/src/*.cu, compiled from
its sources with nvcc, driven by oracle/ref/harness.cu) on seeded inputs; the generating
script is tests/golden/make_fixtures.py.

The CPU tests pin the oracle to those outputs; the GPU tests hold this library's kernels,
called through the C ABI, to the same outputs.  Tolerances:
  * candidate init, f16 packing, radix sort, prune pairs, prune: bit-exact;
  * JFA seed: bit-exact where one site maps to a texel; where several collide, the
    reference keeps whichever write lands last (a race), this library the lowest id --
    the reference's pick must be one of the colliding sites;
  * JFA flood and VPT candidate lists: bit-exact, oracle and GPU (the GPU kernels use the
    reference's FP32 operations in its order; also over chains of passes, below);
  * rendered RGB: oracle <= 2e-6, GPU <= 1e-5 max abs (FMA contraction);
  * autograd adjoint (the reference's render_sad_backward): every entry within 1e-3
    (oracle) / 1e-4 (GPU) of its sum A of absolute pixel terms, and each parameter's
    vector within a relative L2 error of 1e-4; the scale is A, not the entry itself,
    because the reference sums float terms with atomics in no fixed order and entries
    whose terms cancel have no relative accuracy to hold;
  * per-site gradients: relative L2 error per parameter <= 1e-4 (oracle) / 1e-3 (GPU),
    every entry within 1% / 0.5% of its sum of absolute pixel terms (the reference sums
    with float atomics in no fixed order);
  * removal delta 1e-3 relative; tau diffusion and Adam 2e-6; site statistics 2e-4
    relative; densify keys within 2 ulps of the reference's powf; split positions 1e-4
    relative, split axis / anisotropy 1e-2 (eigen-decomposition of a cancellation-prone
    covariance).
"""
import os

import numpy as np
import pytest

from checks import assert_close_sum, assert_grads_close

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
U32 = 0xFFFFFFFF


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def seed_collisions(sites, w, h, ds=1):
    """texel -> ids of the active sites whose seed lands there (jfa.cu seed mapping)."""
    inv = np.float32(1.0) / np.float32(max(ds, 1))
    x = np.clip((sites[:, 0] * inv).astype(np.int64), 0, w - 1)
    y = np.clip((sites[:, 1] * inv).astype(np.int64), 0, h - 1)
    out = {}
    for i in np.nonzero(sites[:, 0] >= 0)[0]:
        out.setdefault(int(y[i] * w + x[i]), []).append(int(i))
    return out


def check_seed(got, ref, cand0_in, sites, w, h, ds):
    col = seed_collisions(sites, w, h, ds)
    np.testing.assert_array_equal(got[:, 1:], ref[:, 1:])
    for p in range(w * h):
        ids = col.get(p)
        if ids is None:
            assert got[p, 0] == ref[p, 0] == cand0_in[p, 0]
        else:
            assert got[p, 0] == min(ids)
            assert ref[p, 0] in ids


def grads_case(name):
    z = load(name)
    w, h, n, rem = (int(v) for v in z["params"])
    return z, w, h, n, bool(rem)


GRAD_CASES = ["grads_plain", "grads_removal", "grads_ssim"]
VPT_CASES = ["vpt_hilbert", "vpt_plain"]
VPT_IDX = (0, 3, 9, 70000)


# ---------------------------------------------------------------------------
# oracle vs reference (CPU)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", ["render_61x37", "render_padded"])
def test_oracle_render(orc, name):
    z = load(name)
    w, h, cw, ch, n = (int(v) for v in z["params"])
    got = orc.render(z["cand0"], z["cand1"], z["sites"], w, h, cw, ch, float(z["inv_s2"]))
    assert np.max(np.abs(got - z["out"])) <= 2e-6


@pytest.mark.parametrize("name", ["init_cand_random", "init_cand_perpixel"])
def test_oracle_init_candidates(orc, name):
    z = load(name)
    n, seed, pp, w, h = (int(v) for v in z["params"])
    a, b = orc.init_candidates(n, seed, pp, w, h)
    np.testing.assert_array_equal(a, z["c0"])
    np.testing.assert_array_equal(b, z["c1"])


def test_oracle_pack(orc):
    z = load("pack")
    np.testing.assert_array_equal(orc.pack_sites(z["sites"]), z["packed"])


def test_oracle_jfa_seed(orc):
    z = load("jfa_seed")
    n, w, h, ds = (int(v) for v in z["params"])
    got = orc.jfa_seed(z["cand0"], z["sites"], w, h, ds)
    check_seed(got, z["out"], z["cand0"], z["sites"], w, h, ds)


def test_oracle_jfa_flood(orc):
    z = load("jfa_flood")
    n, w, h = (int(v) for v in z["params"])
    for step in (32, 4, 1):
        got = orc.jfa_flood(z[f"in_{step}"], z["sites"], step, w, h, 1, None, None, float(z["inv_s2"]))
        np.testing.assert_array_equal(got, z[f"out_{step}"])


@pytest.mark.parametrize("name", VPT_CASES)
def test_oracle_vpt(orc, name):
    z = load(name)
    w, h, n, hil = (int(v) for v in z["params"])
    for idx in VPT_IDX:
        step = orc.pack_jump_step(idx, w, h)
        a, b = orc.vpt_pass(z["cand0"], z["cand1"], z["packed"], n, step, idx >> 16, w, h, 64.0, 0, 4,
                            z["horder"] if hil else None, z["hpos"] if hil else None,
                            1 if hil else 0, 32 if hil else 0)
        np.testing.assert_array_equal(a, z[f"out0_{idx}"])
        np.testing.assert_array_equal(b, z[f"out1_{idx}"])


@pytest.mark.parametrize("name", GRAD_CASES)
def test_oracle_gradients(orc, name):
    z, w, h, n, rem = grads_case(name)
    g, a, r = orc.compute_gradients(z["cand0"], z["cand1"], z["target"], z["sites"], w, h,
                                    rendered=z["rendered"], ssim_weight=float(z["ssim"]), removal=rem)
    assert_grads_close(z["grads"].astype(np.float64), g, a, rel_l2=1e-4, guard=0.01)
    if rem:
        assert np.all(np.abs(z["removal"] - r) <= 1e-3 * np.maximum(np.abs(r), 1.0))


ADJ_CASES = ["knn_64x48", "random_61x37", "knn_97x65"]


def adjoint_case(name):
    z = load("render_backward")
    w, h, n = (int(v) for v in z[f"{name}_params"])
    return ({k: z[f"{name}_{k}"] for k in ("cand0", "cand1", "sites", "grad_out", "grad_sites", "render")},
            w, h, n, float(z[f"{name}_inv_s2"]))


def check_adjoint(got, want, absw, rtol):
    """[N,10] gradients against the reference's: each parameter's vector within 1e-4
    relative L2, every entry within rtol of its absolute-term sum."""
    for k in range(10):
        num = np.linalg.norm(got[:, k] - want[:, k])
        assert num <= 1e-4 * max(np.linalg.norm(want[:, k]), 1e-12), (k, num)
    assert_close_sum(got, want, absw, rtol=rtol, atol=1e-7, what="adjoint")


@pytest.mark.parametrize("name", ADJ_CASES)
def test_oracle_render_backward(orc, name):
    z, w, h, n, inv = adjoint_case(name)
    r = orc.render(z["cand0"], z["cand1"], z["sites"], w, h, inv_s2=inv)
    assert np.max(np.abs(r - z["render"])) <= 2e-6
    g, a = orc.render_backward(z["cand0"], z["cand1"], z["sites"], z["grad_out"], w, h, inv_s2=inv)
    check_adjoint(g, z["grad_sites"].astype(np.float64), a, rtol=1e-3)
    if not name.startswith("knn"):
        return
    # the reference against the FP64 restatement of the same adjoint, on the nearest-site
    # fields a fit sees (a random field's far candidates make single FP32 terms
    # ill-conditioned, in the reference as in any FP32 evaluation)
    g64 = orc.render_backward_d(z["cand0"], z["cand1"], z["sites"].astype(np.float64),
                                z["grad_out"].astype(np.float64), w, h, inv)
    assert_close_sum(z["grad_sites"].astype(np.float64), g64, a, rtol=2e-4, atol=1e-7, what="reference vs FP64")


def test_oracle_tau_diffuse(orc):
    z = load("tau")
    w, h, n = (int(v) for v in z["params"])
    got = orc.tau_diffuse(z["cand0"], z["cand1"], z["sites"], z["raw"], z["gin"], float(z["lam"]), w, h)
    np.testing.assert_allclose(got, z["out"], rtol=2e-6, atol=2e-7)


def test_oracle_adam(orc):
    z = load("adam")
    n, w, h = (int(v) for v in z["params"])
    s, a = orc.adam_update(z["sites"], z["adam"], z["grads"], z["lr"], 0.9, 0.999, 1e-8, int(z["t"]), w, h)
    np.testing.assert_allclose(s, z["sites_out"], rtol=2e-6, atol=2e-6)
    np.testing.assert_allclose(a, z["adam_out"], rtol=2e-6, atol=1e-9)


def sort_names():
    z = load("sort")
    return sorted(k[3:] for k in z.files if k.startswith("in_"))


@pytest.mark.parametrize("case", sort_names())
def test_oracle_radix_sort(orc, case):
    z = load("sort")
    got = orc.radix_sort_pairs(z[f"in_{case}"], int(z[f"maxkey_{case}"]))
    np.testing.assert_array_equal(got, z[f"out_{case}"])


def test_oracle_topology(orc):
    z = load("topology")
    n, pc, w, h, ns, cap, k = (int(v) for v in z["params"])
    np.testing.assert_array_equal(orc.prune_pairs(z["sites"], z["removal"], pc, float(np.float32(1 / 4096))),
                                  z["prune_pairs"])
    np.testing.assert_array_equal(orc.prune_sites(z["sites"], z["prune_idx"]), z["pruned"])
    st = orc.site_stats(z["stats_cand0"], z["stats_cand1"], z["stats_target"], z["stats_sites"], w, h)
    np.testing.assert_allclose(st, z["stats"], rtol=2e-4, atol=1e-4)
    dp = orc.densify_pairs(z["stats_sites"], z["stats"][0], z["stats"][1], ns, 1.0, 0.7)
    np.testing.assert_array_equal(dp[:, 1], z["densify_pairs"][:, 1])
    assert np.all(np.abs(dp[:, 0].astype(np.int64) - z["densify_pairs"][:, 0].astype(np.int64)) <= 2)
    st7 = [z["stats"][i] for i in (0, 2, 3, 4, 5, 6, 7)]
    ss, sa = orc.split_sites(z["split_in"], np.ones((cap, 20), np.float32), z["split_idx"], st7, ns,
                             z["stats_target"], w, h)
    check_split(ss, sa, z)


def check_split(ss, sa, z):
    ang = [7, 8, 9]
    rest = [c for c in range(10) if c not in ang]
    np.testing.assert_allclose(ss[:, rest], z["split_sites"][:, rest], rtol=1e-4, atol=2e-4)
    np.testing.assert_allclose(ss[:, ang], z["split_sites"][:, ang], rtol=1e-2, atol=1e-2)
    np.testing.assert_array_equal(sa, z["split_adam"])


def sha(*arrays):
    import hashlib
    return np.frombuffer(hashlib.sha256(b"".join(np.ascontiguousarray(a).tobytes() for a in arrays)).digest(),
                         np.uint8)


def chain_start(z, floods):
    """(cand0, cand1) entering the first VPT pass: runJFA's ping-pong of the flood
    outputs (sad_cuda.cu:1641-1654).  floods[0] is the seeded field, then one entry per
    flood pass."""
    if (len(floods) - 1) % 2 == 0:
        return floods[-1], floods[-2]
    return floods[-1], floods[-1]


def check_chain(z, flood_fn, vpt_fn):
    """Run the chain with the given pass functions and compare every pass's digest."""
    w, h, n = (int(v) for v in z["params"])
    field, floods = z["seed"], [z["seed"]]
    for s_ in z["jfa_steps"]:
        field = flood_fn(field, int(s_))
        np.testing.assert_array_equal(sha(field), z[f"jfa_{int(s_)}"], err_msg=f"JFA flood step {int(s_)}")
        floods.append(field)
    np.testing.assert_array_equal(field, z["jfa_final"])
    c0, c1 = chain_start(z, floods)
    for i in range(16):
        c0, c1 = vpt_fn(c0, c1, i)
        np.testing.assert_array_equal(sha(c0, c1), z[f"vpt_{i}"], err_msg=f"VPT pass {i}")
    np.testing.assert_array_equal(c0, z["vpt_final0"])
    np.testing.assert_array_equal(c1, z["vpt_final1"])
    return c0, c1


def test_oracle_candidate_chain(orc):
    z = load("cand_chain")
    w, h, n = (int(v) for v in z["params"])
    inv = float(z["inv_s2"])
    np.testing.assert_array_equal(orc.pack_sites(z["sites"]), z["packed"])
    c0, c1 = check_chain(
        z, lambda f, s_: orc.jfa_flood(f, z["sites"], s_, w, h, 1, None, None, inv),
        lambda a, b, i: orc.vpt_pass(a, b, z["packed"], n, orc.pack_jump_step(i, w, h), i >> 16, w, h, 64.0, 0, 4,
                                     z["horder"], z["hpos"], 1, 32))
    assert np.max(np.abs(orc.render(c0, c1, z["sites"], w, h, inv_s2=inv) - z["render"])) <= 2e-6


# ---------------------------------------------------------------------------
# this library's kernels vs reference (GPU, through the C ABI)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def gops(cuda):
    from sad_gb300 import ops
    return ops


def _t():
    import torch
    return torch


def t32(a):
    torch = _t()
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def tf(a):
    torch = _t()
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def u32(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["render_61x37", "render_padded"])
def test_gpu_render(gops, name):
    z = load(name)
    w, h, cw, ch, n = (int(v) for v in z["params"])
    got = gops.render_sad_padded(t32(z["cand0"]), t32(z["cand1"]), tf(z["sites"]), float(z["inv_s2"]),
                                 w, h, cw, ch).cpu().numpy()
    assert np.max(np.abs(got - z["out"])) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["init_cand_random", "init_cand_perpixel"])
def test_gpu_init_candidates(gops, name):
    z = load(name)
    n, seed, pp, w, h = (int(v) for v in z["params"])
    assert bool(pp) == (n == w * h)
    a, b = gops.init_candidates(w, h, n, seed)
    np.testing.assert_array_equal(u32(a), z["c0"])
    np.testing.assert_array_equal(u32(b), z["c1"])


@pytest.mark.gpu
def test_gpu_pack(gops):
    torch = _t()
    z = load("pack")
    n = z["sites"].shape[0]
    packed = torch.zeros((n, 8), dtype=torch.float16, device="cuda")
    gops.pack_candidate_sites(tf(z["sites"]), packed, 0)
    np.testing.assert_array_equal(packed.cpu().numpy().view(np.uint16), z["packed"])


@pytest.mark.gpu
def test_gpu_jfa_seed(gops):
    z = load("jfa_seed")
    n, w, h, ds = (int(v) for v in z["params"])
    got = u32(gops.jfa_seed(t32(z["cand0"]), tf(z["sites"]), 0, ds, w, h))
    check_seed(got, z["out"], z["cand0"], z["sites"], w, h, ds)


@pytest.mark.gpu
def test_gpu_jfa_flood(gops):
    torch = _t()
    z = load("jfa_flood")
    n, w, h = (int(v) for v in z["params"])
    inv = float(z["inv_s2"])
    for step in (32, 4, 1):
        out = torch.empty((w * h, 4), dtype=torch.int32, device="cuda")
        got = u32(gops.jfa_flood(t32(z[f"in_{step}"]), out, tf(z["sites"]), inv, 0, step, 1, w, h))
        np.testing.assert_array_equal(got, z[f"out_{step}"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", VPT_CASES)
def test_gpu_vpt(gops, orc, name):
    torch = _t()
    z = load(name)
    w, h, n, hil = (int(v) for v in z["params"])
    inv = float(z["inv_s2"])
    packed = torch.from_numpy(z["packed"].view(np.float16)).cuda()
    dummy = torch.zeros(1, dtype=torch.int32, device="cuda")
    ho = t32(z["horder"]) if hil else dummy
    hp = t32(z["hpos"]) if hil else dummy
    for idx in VPT_IDX:
        step = orc.pack_jump_step(idx, w, h)
        o0 = torch.empty((w * h, 4), dtype=torch.int32, device="cuda")
        o1 = torch.empty((w * h, 4), dtype=torch.int32, device="cuda")
        gops.update_candidates_compact(t32(z["cand0"]), t32(z["cand1"]), o0, o1, packed, ho, hp, inv, n,
                                       step, idx >> 16, 64.0, 0, 4, 1 if hil else 0, 32 if hil else 0, 1,
                                       w, h, w, h)
        np.testing.assert_array_equal(u32(o0), z[f"out0_{idx}"])
        np.testing.assert_array_equal(u32(o1), z[f"out1_{idx}"])


@pytest.mark.gpu
def test_gpu_candidate_chain(gops):
    """Eight JFA flood passes and sixteen VPT passes chained through this library's
    kernels, bit-exact against the reference pass by pass; then the whole render-from-sites
    path (sad_render_from_sites: its own seed, flood and VPT kernels on prepared site
    records, and the render) against the reference's render of the same chain."""
    import ctypes as C
    torch = _t()
    from sad_gb300 import _lib
    z = load("cand_chain")
    w, h, n = (int(v) for v in z["params"])
    inv = float(z["inv_s2"])
    s_t = tf(z["sites"])
    packed = torch.from_numpy(z["packed"].view(np.float16)).cuda()
    ho, hp = t32(z["horder"]), t32(z["hpos"])

    def flood(f, s_):
        out = torch.empty((w * h, 4), dtype=torch.int32, device="cuda")
        return u32(gops.jfa_flood(t32(f), out, s_t, inv, 0, s_, 1, w, h))

    def vpt(a, b, i):
        o0 = torch.empty((w * h, 4), dtype=torch.int32, device="cuda")
        o1 = torch.empty((w * h, 4), dtype=torch.int32, device="cuda")
        gops.update_candidates_compact(t32(a), t32(b), o0, o1, packed, ho, hp, inv, n,
                                       int(np.uint32(_lib.load().sad_pack_jump_step(i, w, h))), i >> 16,
                                       64.0, 0, 4, 1, 32, 1, w, h, w, h)
        return u32(o0), u32(o1)

    seeded = u32(gops.jfa_seed(t32(np.full((w * h, 4), U32, np.uint32)), s_t, 0, 1, w, h))
    np.testing.assert_array_equal(seeded, z["seed"])
    check_chain(z, flood, vpt)

    lib = _lib.load()
    cfg = _lib.RenderConfig()
    lib.sad_render_config_default(C.byref(cfg))
    assert (cfg.candidate_passes, cfg.use_jfa, cfg.jfa_rounds, cfg.cand_inject_count, cfg.cand_hilbert_probes,
            cfg.cand_hilbert_window, cfg.cand_radius_probes) == (16, 1, 1, 4, 1, 32, 0)
    nb = lib.sad_render_scratch_bytes(n, w, h, 1)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    out = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    assert lib.sad_render_from_sites(C.byref(cfg), C.c_void_p(s_t.data_ptr()), n, w, h, C.c_void_p(out.data_ptr()),
                                     C.c_void_p(scratch.data_ptr()), nb, None) == 0, lib.sad_last_error()
    torch.cuda.synchronize()
    assert np.max(np.abs(out.cpu().numpy() - z["render"])) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", GRAD_CASES)
def test_gpu_gradients(gops, orc, name):
    torch = _t()
    z, w, h, n, rem = grads_case(name)
    bufs = [torch.zeros(n, dtype=torch.float32, device="cuda") for _ in range(11)]
    gops.compute_gradients_tiled(t32(z["cand0"]), t32(z["cand1"]), tf(z["target"]), tf(z["rendered"]),
                                 tf(np.ones((h, w), np.float32)), tf(z["sites"]), *bufs, float(z["inv_s2"]),
                                 0, int(rem), float(z["ssim"]), w, h)
    _, a, _ = orc.compute_gradients(z["cand0"], z["cand1"], z["target"], z["sites"], w, h,
                                    rendered=z["rendered"], ssim_weight=float(z["ssim"]), removal=rem)
    got = np.stack([b.cpu().numpy() for b in bufs[:10]]).astype(np.float64)
    assert_grads_close(got, z["grads"].astype(np.float64), a)
    if rem:
        r = bufs[10].cpu().numpy()
        assert np.all(np.abs(r - z["removal"]) <= 1e-3 * np.maximum(np.abs(z["removal"]), 1.0))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ADJ_CASES)
def test_gpu_render_backward(gops, orc, name):
    """torch.ops.sad.render_sad_backward (this library's adjoint kernel) against the
    reference's render_sad_backward on the same inputs."""
    z, w, h, n, inv = adjoint_case(name)
    got = gops.render_sad_backward(t32(z["cand0"]), t32(z["cand1"]), tf(z["sites"]), tf(z["grad_out"]),
                                   inv, w, h).cpu().numpy().astype(np.float64)
    _, a = orc.render_backward(z["cand0"], z["cand1"], z["sites"], z["grad_out"], w, h, inv_s2=inv)
    check_adjoint(got, z["grad_sites"].astype(np.float64), a, rtol=1e-4)
    img = gops.render_sad(t32(z["cand0"]), t32(z["cand1"]), tf(z["sites"]), inv, w, h).cpu().numpy()
    assert np.max(np.abs(img - z["render"])) <= 1e-5


@pytest.mark.gpu
def test_gpu_tau_diffuse(gops):
    torch = _t()
    z = load("tau")
    w, h, n = (int(v) for v in z["params"])
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    gops.tau_diffuse(t32(z["cand0"]), t32(z["cand1"]), tf(z["sites"]), tf(z["raw"]), tf(z["gin"]), out, 0,
                     float(z["lam"]), 1, w, h)
    np.testing.assert_allclose(out.cpu().numpy(), z["out"], rtol=2e-6, atol=2e-7)


@pytest.mark.gpu
def test_gpu_adam(gops):
    z = load("adam")
    n, w, h = (int(v) for v in z["params"])
    s_t, a_t = tf(z["sites"]), tf(z["adam"])
    gops.adam_update(s_t, a_t, *[tf(g) for g in z["grads"]], *[float(x) for x in z["lr"]], 0.9, 0.999,
                     1e-8, int(z["t"]), w, h)
    np.testing.assert_allclose(s_t.cpu().numpy(), z["sites_out"], rtol=2e-6, atol=2e-6)
    np.testing.assert_allclose(a_t.cpu().numpy(), z["adam_out"], rtol=2e-6, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("case", sort_names())
def test_gpu_radix_sort(gops, case):
    z = load("sort")
    p = t32(z[f"in_{case}"])
    gops.radix_sort_pairs(p, int(z[f"maxkey_{case}"]))
    np.testing.assert_array_equal(u32(p), z[f"out_{case}"])


@pytest.mark.gpu
def test_gpu_topology(gops):
    torch = _t()
    z = load("topology")
    n, pc, w, h, ns, cap, k = (int(v) for v in z["params"])
    pairs = torch.zeros((pc, 2), dtype=torch.int32, device="cuda")
    gops.compute_prune_score_pairs(tf(z["sites"]), tf(z["removal"]), pairs, 0, float(np.float32(1 / 4096)), pc)
    np.testing.assert_array_equal(u32(pairs), z["prune_pairs"])
    s_t = tf(z["sites"])
    gops.prune_sites(s_t, t32(z["prune_idx"]), z["prune_idx"].shape[0])
    np.testing.assert_array_equal(s_t.cpu().numpy(), z["pruned"])
    st = [torch.zeros(ns, dtype=torch.float32, device="cuda") for _ in range(8)]
    gops.compute_site_stats_tiled(t32(z["stats_cand0"]), t32(z["stats_cand1"]), tf(z["stats_target"]),
                                  tf(np.ones((h, w), np.float32)), tf(z["stats_sites"]), *st,
                                  float(np.float32(1.0 / w ** 2)), ns, w, h)
    got = np.stack([s.cpu().numpy() for s in st])
    np.testing.assert_allclose(got, z["stats"], rtol=2e-4, atol=1e-4)
    dp = torch.zeros((ns, 2), dtype=torch.int32, device="cuda")
    gops.compute_densify_score_pairs(tf(z["stats_sites"]), tf(z["stats"][0]), tf(z["stats"][1]), dp, ns,
                                     1.0, 0.7, ns)
    dp = u32(dp)
    np.testing.assert_array_equal(dp[:, 1], z["densify_pairs"][:, 1])
    assert np.all(np.abs(dp[:, 0].astype(np.int64) - z["densify_pairs"][:, 0].astype(np.int64)) <= 2)
    s_t, a_t = tf(z["split_in"]), tf(np.ones((cap, 20), np.float32))
    st7 = [z["stats"][i] for i in (0, 2, 3, 4, 5, 6, 7)]
    gops.split_sites(s_t, a_t, t32(z["split_idx"]), *[tf(x) for x in st7], ns, k, tf(z["stats_target"]))
    check_split(s_t.cpu().numpy(), a_t.cpu().numpy(), z)
