"""Seeded test inputs shared by the CPU and GPU tests.

Sort cases restate the case list of the reference's radix-sort program
(backends/metal/tests/test_sort.swift:123-423, 827-907): random keys, float-derived
descending keys, small / non-power-of-two / block-boundary counts, identical keys,
byte-boundary key ranges, sorted and reversed input, bit patterns and the 2-vs-4-pass
boundary, each with the program's seed and its xorshift64* generator
(test_sort.swift:18-37).  Inputs are padded to the next power of two with
(0xFFFFFFFF, 0xFFFFFFFF) as the program does; the expected result is the stable sort by
key (masked to 16 bits when 2 passes are used).
"""
from __future__ import annotations

import numpy as np

U32 = 0xFFFFFFFF


class XorShift64Star:
    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF or 0x123456789ABCDEF0

    def u32(self) -> int:
        x = self.s
        x ^= x >> 12
        x ^= (x << 25) & 0xFFFFFFFFFFFFFFFF
        x ^= x >> 27
        self.s = x
        return ((x * 2685821657736338717) & 0xFFFFFFFFFFFFFFFF) >> 32

    def f01(self) -> float:
        return float(np.float32(self.u32() & 0x00FFFFFF) / np.float32(0x01000000))


def next_pow2(n: int) -> int:
    p = 1
    while p < n:
        p <<= 1
    return p


def _pairs(keys) -> np.ndarray:
    k = np.asarray(keys, dtype=np.uint64).astype(np.uint32)
    return np.stack([k, np.arange(len(k), dtype=np.uint32)], axis=1)


def _pad(p: np.ndarray) -> np.ndarray:
    n = next_pow2(p.shape[0])
    if n == p.shape[0]:
        return p
    pad = np.full((n - p.shape[0], 2), U32, dtype=np.uint32)
    return np.concatenate([p, pad])


def _random(count, key_max, seed):
    r = XorShift64Star(seed)
    return [r.u32() if key_max == U32 else r.u32() % max(1, key_max) for _ in range(count)]


def sort_cases(include_large: bool = False):
    """Yields (name, padded pairs [M,2] u32, max_key_exclusive, count)."""
    out = []
    for km in (10_000, U32):
        out.append((f"random_k{km}", _pad(_pairs(_random(4096, km, 0xC0FFEE))), km, 4096))
    r = XorShift64Star(0xBADC0DE)
    fk = []
    for _ in range(4096):
        e = r.f01() * 20.0 - 10.0
        score = np.float32((2.0 ** e) * r.f01())
        fk.append(U32 - int(np.float32(score).view(np.uint32)))
    out.append(("float_desc", _pad(_pairs(fk)), U32, 4096))
    for c in (1, 2, 3, 4, 7, 8, 15, 16, 17, 31, 32, 33, 63, 64, 65, 127, 128, 255, 256, 257):
        out.append((f"small_{c}", _pad(_pairs(_random(c, U32, c))), U32, c))
    for c in (256, 1024, 4096):
        for kv in (0, 1, 255, 256, 65535, 65536, U32 - 1):
            mk = kv + 1 if kv < (1 << 16) else U32
            out.append((f"same_{c}_{kv}", _pad(_pairs([kv] * c)), mk, c))
    for name, lo, hi in (("b255", 250, 260), ("b65535", 65530, 65542),
                         ("b2_24", 16777210, 16777222), ("low", 0, 10), ("high", U32 - 100, U32)):
        rr = XorShift64Star(0xDEAD)
        size = hi - lo + 1
        keys = [lo + rr.u32() % size for _ in range(4096)]
        mk = hi + 1 if hi < (1 << 16) else U32
        out.append((f"range_{name}", _pad(_pairs(keys)), mk, 4096))
    for c in (256, 1024, 2048):
        mk = c if c <= 65536 else U32
        out.append((f"sorted_{c}", _pad(_pairs(range(c))), mk, c))
        out.append((f"reversed_{c}", _pad(_pairs(range(c - 1, -1, -1))), mk, c))
    for c in (100, 200, 300, 500, 700, 900, 1000, 1023, 1025, 1100, 2000, 2047, 2049, 3000, 4000,
              4095, 4097, 5000, 10000, 16383, 16385):
        out.append((f"npow2_{c}", _pad(_pairs(_random(c, U32, c ^ 0xCAFE))), U32, c))
    for pat in ("alternating", "low", "high", "samehigh"):
        rr = XorShift64Star(0xDA77E8)
        keys = []
        for i in range(1024):
            if pat == "alternating":
                keys.append(rr.u32() if i % 2 == 0 else U32 - rr.u32())
            elif pat == "low":
                keys.append(rr.u32() & 0x0000FFFF)
            elif pat == "high":
                keys.append(rr.u32() & 0xFFFF0000)
            else:
                keys.append(0xABCD0000 | (rr.u32() & 0x0000FFFF))
        out.append((f"pattern_{pat}", _pad(_pairs(keys)), U32, 1024))
    for c in (512, 1024, 1025, 2048, 2049, 3072, 4096, 5000, 8192, 10240):
        out.append((f"grid_{c}", _pad(_pairs(_random(c, U32, c ^ 0xBEEF))), U32, c))
    for mk in (1 << 15, 1 << 16, (1 << 16) + 1, 1 << 17, 1 << 24, U32):
        out.append((f"passes_{mk}", _pad(_pairs(_random(4096, mk, mk ^ 0xABCD))), mk, 4096))
    if include_large:
        rr = XorShift64Star(0xF1E1D)
        n = 256 * 256 * 8
        keys = np.array([rr.u32() % 1000 for _ in range(n)], dtype=np.uint32)
        out.append(("pipeline_256sq", _pad(_pairs(keys)), 1000, n))
    return out


def expected_sort(pairs: np.ndarray, max_key_exclusive: int) -> np.ndarray:
    mask = 0xFFFF if max_key_exclusive <= 65536 else U32
    order = np.argsort(pairs[:, 0] & np.uint32(mask), kind="stable")
    return pairs[order]


def scene(w: int, h: int, n: int, seed: int = 0):
    """(image [H,W,3], sites [N,10]) from the synthetic generators."""
    import sad_gb300.synthetic as syn
    img = syn.synthetic_image(w, h, seed=seed)
    return img, syn.synthetic_sites(img, n, seed=seed)


def random_field(w: int, h: int, n: int, seed: int, empty_frac: float = 0.05, dup_frac: float = 0.05,
                 invalid_frac: float = 0.02):
    """Candidate field with random ids and the edge cases the kernels must handle: empty
    slots (0xFFFFFFFF), ids >= n, and duplicated ids within a list."""
    rng = np.random.default_rng(seed)
    ids = rng.integers(0, n, size=(w * h, 8), dtype=np.int64).astype(np.uint32)
    m = rng.random((w * h, 8))
    ids[m < empty_frac] = U32
    bad = (m >= empty_frac) & (m < empty_frac + invalid_frac)
    ids[bad] = n + rng.integers(0, 100, size=int(bad.sum()), dtype=np.int64).astype(np.uint32)
    dup = rng.random(w * h) < dup_frac
    ids[dup, 7] = ids[dup, 0]
    return np.ascontiguousarray(ids[:, :4]), np.ascontiguousarray(ids[:, 4:])


def knn_field(sites: np.ndarray, w: int, h: int, k: int = 8):
    """Candidate field of each pixel's k nearest sites (Euclidean), a realistic field."""
    from scipy.spatial import cKDTree
    tree = cKDTree(sites[:, :2].astype(np.float64))
    yy, xx = np.mgrid[0:h, 0:w]
    pts = np.stack([xx.ravel(), yy.ravel()], axis=1).astype(np.float64)
    _, idx = tree.query(pts, k=k)
    idx = idx.astype(np.uint32)
    return np.ascontiguousarray(idx[:, :4]), np.ascontiguousarray(idx[:, 4:])


def oracle_render_from_sites(orc, sites, w, h, passes=16, inject=4, hprobes=1, hwin=32):
    """renderVoronoiFromSites: clear, seed, flood (ping-pong inside the field), VPT passes."""
    n = sites.shape[0]
    inv = 1.0 / max(w, h) ** 2
    a0 = np.full((w * h, 4), 0xFFFFFFFF, np.uint32)
    a1 = a0.copy()
    a0 = orc.jfa_seed(a0, sites, w, h)
    step = 1
    while step < max(w, h):
        step <<= 1
    src, dst = a0, a1
    s = step // 2
    while s >= 1:
        dst = orc.jfa_flood(src, sites, s, w, h)
        src, dst = dst, src
        s //= 2
    a0, a1 = src, dst
    packed = orc.pack_sites(sites)
    bits = orc.hilbert_bits_for_size(w, h)
    padded = (n + 1023) // 1024 * 1024
    pairs = orc.radix_sort_pairs(orc.hilbert_pairs(sites, padded, w, h, bits),
                                 0xFFFFFFFF if bits >= 16 else 1 << (2 * bits))
    horder, hpos = orc.hilbert_order(pairs, n)
    for i in range(passes):
        a0, a1 = orc.vpt_pass(a0, a1, packed, n, orc.pack_jump_step(i, w, h), i >> 16, w, h, 64.0, 0,
                              inject, horder, hpos, hprobes, hwin)
    return orc.render(a0, a1, sites, w, h), (a0, a1)
