"""Generate golden fixtures from the reference's own CUDA kernels.

    oracle/ref/stage.sh /path/to/reference     # copy its sources to baseline/_ref/ (git-ignored)
    oracle/ref/build.sh                        # nvcc -> oracle/_ref/ref_harness (needs a GPU to run)
    python tests/golden/make_fixtures.py [outdir] [--only=chains]

Each case writes seeded inputs to a scratch directory, runs one reference kernel through
oracle/_ref/ref_harness, and stores inputs + the reference's outputs in <outdir>/<case>.npz
(default: tests/golden/).  Inputs avoid the reference's undefined behaviour: masks are all
ones for the gradient kernel (its masked pixels return before a barrier).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle")]
import cases  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
U32 = 0xFFFFFFFF


def run(cmd, d, *scalars):
    args = [HARNESS, cmd, d] + [repr(float(s)) if isinstance(s, float) else str(int(s)) for s in scalars]
    subprocess.run(args, check=True)


def put(d, name, arr):
    np.ascontiguousarray(arr).tofile(os.path.join(d, name + ".bin"))


def get(d, name, dtype, shape):
    return np.fromfile(os.path.join(d, name + ".bin"), dtype=dtype).reshape(shape)


def f32s(x: float) -> float:
    return float(np.float32(x))


def main(outdir: str):
    os.makedirs(outdir, exist_ok=True)
    import orc
    tmp = tempfile.mkdtemp()

    def save(name, **arrays):
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **arrays)
        print("wrote", name)

    # render (full-resolution and padded candidate fields)
    for name, (w, h, cw, ch, n, seed) in {"render_61x37": (61, 37, 61, 37, 300, 1),
                                          "render_padded": (96, 64, 48, 32, 500, 2)}.items():
        img, sites = cases.scene(w, h, n, seed)
        sites[::13, 0] = -1.0
        c0, c1 = cases.random_field(cw, ch, n, seed)
        inv = f32s(1.0 / max(w, h) ** 2)
        for k, v in (("cand0", c0), ("cand1", c1), ("sites", sites)):
            put(tmp, k, v)
        run("render", tmp, n, w, h, cw, ch, inv)
        save(name, cand0=c0, cand1=c1, sites=sites, out=get(tmp, "out", np.float32, (h, w, 3)),
             params=np.array([w, h, cw, ch, n], np.int64), inv_s2=np.float32(inv))

    # candidate init (random and per-pixel)
    for name, (n, seed, pp, w, h) in {"init_cand_random": (1000, 12345, 0, 40, 24),
                                      "init_cand_perpixel": (200, 7, 1, 20, 10)}.items():
        run("init_cand", tmp, n, seed, pp, w, h)
        save(name, c0=get(tmp, "c0", np.uint32, (w * h, 4)), c1=get(tmp, "c1", np.uint32, (w * h, 4)),
             params=np.array([n, seed, pp, w, h], np.int64))

    # f16 packing
    img, sites = cases.scene(64, 64, 3000, 3)
    sites[::7, 0] = -1
    sites[1, :] = [65519.99, 1e-9, 1e5, -3, 1, 1, 1, 0.3, -0.2, 7.0]
    sites[2, :] = [6.1e-5, 2.9802326e-8, -7.5, 0.1, 0, 0, 0, -1.0, 1e-7, -4.0]
    put(tmp, "sites", sites)
    run("pack", tmp, 3000)
    save("pack", sites=sites, packed=get(tmp, "packed", np.uint16, (3000, 8)))

    # JFA seed (collisions) and flood passes
    w, h, n = 40, 30, 900
    img, sites = cases.scene(w, h, n, 4)
    sites[::5, 0] = -1
    c0 = np.random.default_rng(0).integers(0, n, (w * h, 4)).astype(np.uint32)
    put(tmp, "cand0", c0)
    put(tmp, "sites", sites)
    run("jfa_seed", tmp, n, w, h, 1)
    save("jfa_seed", cand0=c0, sites=sites, out=get(tmp, "out", np.uint32, (w * h, 4)),
         params=np.array([n, w, h, 1], np.int64))
    w, h, n = 80, 56, 600
    img, sites = cases.scene(w, h, n, 5)
    sites[::9, 0] = -1
    inv = f32s(1.0 / max(w, h) ** 2)
    field = orc.jfa_seed(np.full((w * h, 4), U32, np.uint32), sites, w, h)
    outs = {}
    for step in (32, 4, 1):
        put(tmp, "cand0", field)
        put(tmp, "sites", sites)
        run("jfa_flood", tmp, n, step, inv, w, h, 1, w, h)
        outs[f"out_{step}"] = get(tmp, "out", np.uint32, (w * h, 4))
        outs[f"in_{step}"] = field.copy()
        field = orc.jfa_flood(field, sites, step, w, h)
    save("jfa_flood", sites=sites, params=np.array([n, w, h], np.int64), inv_s2=np.float32(inv), **outs)

    # VPT passes (with and without Hilbert probes)
    for name, (w, h, n, hil, seed) in {"vpt_hilbert": (96, 64, 800, 1, 10),
                                       "vpt_plain": (50, 50, 300, 0, 12)}.items():
        img, sites = cases.scene(w, h, n, seed)
        sites[::10, 0] = -1
        c0, c1 = cases.random_field(w, h, n, seed)
        packed = orc.pack_sites(sites)
        inv = f32s(1.0 / max(w, h) ** 2)
        bits = orc.hilbert_bits_for_size(w, h)
        padded = (n + 1023) // 1024 * 1024
        pairs = orc.radix_sort_pairs(orc.hilbert_pairs(sites, padded, w, h, bits),
                                     0xFFFFFFFF if bits >= 16 else 1 << (2 * bits))
        horder, hpos = orc.hilbert_order(pairs, n)
        arrays = dict(cand0=c0, cand1=c1, sites=sites, packed=packed, horder=horder, hpos=hpos,
                      params=np.array([w, h, n, hil], np.int64), inv_s2=np.float32(inv))
        for idx in (0, 3, 9, 70000):
            step = orc.pack_jump_step(idx, w, h)
            for k, v in (("cand0", c0), ("cand1", c1), ("packed", packed), ("horder", horder), ("hpos", hpos)):
                put(tmp, k, v)
            run("vpt", tmp, n, step, inv, idx >> 16, 64.0, 0, 4, hil, 32 if hil else 0, 1, w, h, w, h)
            arrays[f"out0_{idx}"] = get(tmp, "out0", np.uint32, (w * h, 4))
            arrays[f"out1_{idx}"] = get(tmp, "out1", np.uint32, (w * h, 4))
        save(name, **arrays)

    # fused gradients (all-ones mask), with removal, with SSIM
    for name, (w, h, n, rem, ssim, seed) in {"grads_plain": (64, 48, 400, 0, 0.0, 20),
                                             "grads_removal": (97, 61, 900, 1, 0.0, 21),
                                             "grads_ssim": (72, 40, 300, 0, 0.2, 22)}.items():
        img, sites = cases.scene(w, h, n, seed)
        sites[::9, 0] = -1
        c0, c1 = cases.knn_field(sites, w, h) if seed != 21 else cases.random_field(w, h, n, seed)
        mask = np.ones((h, w), np.float32)
        rendered = orc.render(c0, c1, sites, w, h)
        inv = f32s(1.0 / max(w, h) ** 2)
        for k, v in (("cand0", c0), ("cand1", c1), ("target", img), ("rendered", rendered),
                     ("mask", mask), ("sites", sites)):
            put(tmp, k, v)
        run("grads", tmp, n, inv, rem, ssim, w, h, w, h)
        g = np.stack([get(tmp, f"g{k}", np.float32, (n,)) for k in range(10)])
        save(name, cand0=c0, cand1=c1, target=img, rendered=rendered, sites=sites, grads=g,
             removal=get(tmp, "removal", np.float32, (n,)),
             params=np.array([w, h, n, rem], np.int64), ssim=np.float32(ssim), inv_s2=np.float32(inv))

    # tau diffusion
    w, h, n = 64, 48, 700
    img, sites = cases.scene(w, h, n, 30)
    sites[::6, 0] = -1
    c0, c1 = cases.random_field(w, h, n, 30)
    rng = np.random.default_rng(0)
    raw = rng.normal(size=n).astype(np.float32)
    gin = rng.normal(size=n).astype(np.float32)
    for k, v in (("cand0", c0), ("cand1", c1), ("sites", sites), ("raw", raw), ("gin", gin)):
        put(tmp, k, v)
    run("tau", tmp, n, 0.037, w, h, 1)
    save("tau", cand0=c0, cand1=c1, sites=sites, raw=raw, gin=gin, out=get(tmp, "out", np.float32, (n,)),
         params=np.array([w, h, n], np.int64), lam=np.float32(0.037))

    # Adam
    n, w, h = 1000, 200, 150
    img, sites = cases.scene(w, h, n, 31)
    sites[::8, 0] = -1
    rng = np.random.default_rng(1)
    grads = rng.normal(size=(10, n)).astype(np.float32) * 50
    adam = (rng.random((n, 20)) * 1e-3).astype(np.float32)
    lr = [0.025, 0.01, 0.01, 0.01, 0.0025, 0.025]
    put(tmp, "sites", sites)
    put(tmp, "adam", adam)
    for k in range(10):
        put(tmp, f"g{k}", grads[k])
    run("adam", tmp, n, *lr, 0.9, 0.999, 1e-8, 7, w, h)
    save("adam", sites=sites, adam=adam, grads=grads, lr=np.float32(lr), t=np.int64(7),
         params=np.array([n, w, h], np.int64), sites_out=get(tmp, "sites_out", np.float32, (n, 10)),
         adam_out=get(tmp, "adam_out", np.float32, (n, 20)))

    # radix sort
    picks = {"random_k4294967295", "random_k10000", "float_desc", "npow2_5000", "passes_65536",
             "passes_65537", "same_4096_65535", "range_b65535", "grid_2049"}
    arrays = {}
    for name, pairs, mk, count in cases.sort_cases():
        if name not in picks:
            continue
        put(tmp, "pairs", pairs)
        run("sort", tmp, pairs.shape[0], mk)
        arrays[f"in_{name}"] = pairs
        arrays[f"out_{name}"] = get(tmp, "out", np.uint32, pairs.shape)
        arrays[f"maxkey_{name}"] = np.int64(mk)
    save("sort", **arrays)

    # score pairs, prune, split, site statistics
    n, pc = 3000, 3072
    img, sites = cases.scene(64, 64, n, 40)
    sites[::10, 0] = -1
    rem = np.random.default_rng(5).normal(size=n).astype(np.float32)
    rem[::17] = np.inf
    put(tmp, "sites", sites)
    put(tmp, "removal", rem)
    run("prune_pairs", tmp, n, f32s(1.0 / 4096), pc)
    pp = get(tmp, "pairs", np.uint32, (pc, 2))
    w, h, ns = 96, 80, 600
    img2, s2 = cases.scene(w, h, ns, 41)
    c0, c1 = cases.knn_field(s2, w, h)
    for k, v in (("cand0", c0), ("cand1", c1), ("target", img2), ("mask", np.ones((h, w), np.float32)),
                 ("sites", s2)):
        put(tmp, k, v)
    run("stats", tmp, ns, f32s(1.0 / w ** 2), w, h, w, h)
    st = np.stack([get(tmp, f"st{k}", np.float32, (ns,)) for k in range(8)])
    put(tmp, "mass", st[0])
    put(tmp, "energy", st[1])
    run("densify_pairs", tmp, ns, 1.0, 0.7, ns)
    dp = get(tmp, "pairs", np.uint32, (ns, 2))
    cap, k = ns + 100, 50
    big = np.zeros((cap, 10), np.float32)
    big[:ns] = s2
    adam = np.ones((cap, 20), np.float32)
    idx = np.arange(0, 2 * k, 2, dtype=np.uint32)
    stats7 = [st[0], st[2], st[3], st[4], st[5], st[6], st[7]]
    put(tmp, "sites", big)
    put(tmp, "adam", adam)
    put(tmp, "idx", idx)
    put(tmp, "target", img2)
    for j, v in enumerate(stats7):
        put(tmp, f"st{j}", v)
    run("split", tmp, cap, k, ns, w, h)
    split_sites = get(tmp, "sites_out", np.float32, (cap, 10))
    split_adam = get(tmp, "adam_out", np.float32, (cap, 20))
    put(tmp, "sites", sites)
    pidx = orc.radix_sort_pairs(pp, U32)[:200, 1].copy()
    put(tmp, "idx", pidx)
    run("prune", tmp, 200)
    save("topology", sites=sites, removal=rem, prune_pairs=pp, prune_idx=pidx,
         pruned=get(tmp, "sites_out", np.float32, (n, 10)), stats_cand0=c0, stats_cand1=c1,
         stats_target=img2, stats_sites=s2, stats=st, densify_pairs=dp, split_in=big, split_idx=idx,
         split_sites=split_sites, split_adam=split_adam, params=np.array([n, pc, w, h, ns, cap, k], np.int64))


def chains(outdir: str):
    """Chains of candidate passes through the reference, recorded pass by pass
    (cand_chain.npz): the render-from-sites build of renderVoronoiFromSites
    (backends/cuda/src/sad_cuda.cu:1616-1655, 1774-1812) -- JFA flood passes from the
    seeded field down to step 1 (ping-ponging as runJFA does, so the first VPT pass sees
    an intermediate field in slots 4-7), then 16 VPT passes with Hilbert probes, 4
    injections and the render -- on a 200x152
    image with 3000 sites.  The seed comes from the oracle (lowest id per texel; the
    reference's seed store is a race), and so do the packed sites and Hilbert order, which
    have fixtures of their own.  Each pass's output is recorded as a SHA-256 digest (the
    final JFA and VPT fields in full), so a difference is located at the first pass it
    appears in."""
    import hashlib

    def digest(*a):
        return np.frombuffer(hashlib.sha256(b"".join(np.ascontiguousarray(x).tobytes() for x in a)).digest(),
                             np.uint8)
    import orc
    tmp = tempfile.mkdtemp()
    w, h, n = 200, 152, 3000
    img, sites = cases.scene(w, h, n, 60)
    sites[::13, 0] = -1
    inv = f32s(1.0 / max(w, h) ** 2)
    field = orc.jfa_seed(np.full((w * h, 4), U32, np.uint32), sites, w, h)
    arrays = dict(sites=sites, seed=field.copy(), params=np.array([w, h, n], np.int64),
                  inv_s2=np.float32(inv))
    step = 1
    while step < max(w, h):
        step <<= 1
    steps, fields = [], [field]
    s_ = step // 2
    while s_ >= 1:
        put(tmp, "cand0", field)
        put(tmp, "sites", sites)
        run("jfa_flood", tmp, n, s_, inv, w, h, 1, w, h)
        field = get(tmp, "out", np.uint32, (w * h, 4))
        arrays[f"jfa_{s_}"] = digest(field)
        fields.append(field)
        steps.append(s_)
        s_ //= 2
    arrays["jfa_steps"] = np.array(steps, np.int64)
    arrays["jfa_final"] = field.copy()
    packed = orc.pack_sites(sites)
    bits = orc.hilbert_bits_for_size(w, h)
    padded = (n + 1023) // 1024 * 1024
    pairs = orc.radix_sort_pairs(orc.hilbert_pairs(sites, padded, w, h, bits),
                                 0xFFFFFFFF if bits >= 16 else 1 << (2 * bits))
    horder, hpos = orc.hilbert_order(pairs, n)
    arrays.update(packed=packed, horder=horder, hpos=hpos)
    # runJFA's ping-pong (sad_cuda.cu:1641-1654): after an even number of passes slots 4-7
    # hold the second-last pass's lists; after an odd number both halves hold the last
    c0 = field
    c1 = fields[-2] if len(steps) % 2 == 0 else field
    for i in range(16):
        st = orc.pack_jump_step(i, w, h)
        for k, v in (("cand0", c0), ("cand1", c1), ("packed", packed), ("horder", horder), ("hpos", hpos)):
            put(tmp, k, v)
        run("vpt", tmp, n, st, inv, i >> 16, 64.0, 0, 4, 1, 32, 1, w, h, w, h)
        c0 = get(tmp, "out0", np.uint32, (w * h, 4))
        c1 = get(tmp, "out1", np.uint32, (w * h, 4))
        arrays[f"vpt_{i}"] = digest(c0, c1)
    arrays["vpt_final0"], arrays["vpt_final1"] = c0.copy(), c1.copy()
    put(tmp, "cand0", c0)
    put(tmp, "cand1", c1)
    put(tmp, "sites", sites)
    run("render", tmp, n, w, h, w, h, inv)
    arrays["render"] = get(tmp, "out", np.float32, (h, w, 3))
    np.savez_compressed(os.path.join(outdir, "cand_chain.npz"), **arrays)
    print("wrote cand_chain")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    out = args[0] if args else HERE
    if "--only=chains" in sys.argv:  # the pass-by-pass chains alone
        os.makedirs(out, exist_ok=True)
        chains(out)
    else:
        main(out)
        chains(out)
