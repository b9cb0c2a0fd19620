"""Baseline JPEG writer for test inputs (ITU-T T.81 sequential DCT, Huffman coded), plus the
exact decode that a conforming reader must produce from the coefficients it wrote.

Test infrastructure only: it builds files that exercise the command-line host's JPEG reader
(sad_gb300/cli/jpeg.cpp) over grey and YCbCr images, the 4:4:4 / 4:2:2 / 4:4:0 / 4:2:0
sampling layouts, 8- and 16-bit quantisation tables, restart intervals and several segment
layouts.  Huffman tables are built per image from symbol counts, quantisation tables are
generated here (no standard tables are reproduced).
"""
from __future__ import annotations

import heapq
import struct

import numpy as np


def zigzag() -> np.ndarray:
    """Natural (row*8+col) index of each zig-zag position (T.81 Figure 5)."""
    out = []
    for s in range(15):
        cells = [(r, s - r) for r in range(max(0, s - 7), min(s, 7) + 1)]
        if s % 2 == 0:
            cells.reverse()  # even anti-diagonals run from bottom-left to top-right
        out.extend(r * 8 + c for r, c in cells)
    return np.array(out)


ZZ = zigzag()
_X = np.arange(8)
BASIS = np.where(_X[None, :] == 0, np.sqrt(0.125), 0.5) * np.cos((2 * _X[:, None] + 1) * _X[None, :] * np.pi / 16)
# BASIS[x, u] = C(u)/2 cos((2x+1) u pi / 16): forward F = B^T f B, inverse f = B F B^T


def quant_table(base: float, slope: float) -> np.ndarray:
    """Natural-order 8x8 table growing with spatial frequency."""
    r, c = np.meshgrid(np.arange(8), np.arange(8), indexing="ij")
    return np.clip(np.rint(base * (1.0 + slope * (r + c))), 1, 65535).astype(np.int64).reshape(64)


def rgb_to_ycbcr(rgb: np.ndarray) -> np.ndarray:
    r, g, b = (rgb[..., k].astype(np.float64) for k in range(3))
    y = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128.0
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128.0
    return np.stack([y, cb, cr], -1)


def _pad_edge(a: np.ndarray, h: int, w: int) -> np.ndarray:
    return np.pad(a, ((0, h - a.shape[0]), (0, w - a.shape[1])), mode="edge")


def _code_lengths(freq: dict[int, int]) -> dict[int, int]:
    """Huffman code lengths for the used symbols, at most 16 bits, never the all-ones code."""
    syms = dict(freq)
    syms[256] = 0  # reserved leaf: takes the all-ones code and is dropped
    heap = [(f, s, [s]) for s, f in syms.items()]
    heapq.heapify(heap)
    depth = {s: 0 for s in syms}
    while len(heap) > 1:
        f1, k1, a = heapq.heappop(heap)
        f2, k2, b = heapq.heappop(heap)
        for s in a + b:
            depth[s] += 1
        heapq.heappush(heap, (f1 + f2, min(k1, k2), a + b))
    del depth[256]
    if max(depth.values()) > 16:
        n = len(depth)
        flat = int(np.ceil(np.log2(n + 1)))
        depth = {s: flat for s in depth}
    return depth


class Huffman:
    def __init__(self, freq: dict[int, int]):
        lengths = _code_lengths(freq)
        self.order = sorted(lengths, key=lambda s: (lengths[s], s))
        self.counts = [0] * 17
        for s in self.order:
            self.counts[lengths[s]] += 1
        self.codes = {}
        code, k = 0, 0
        for l in range(1, 17):
            for _ in range(self.counts[l]):
                self.codes[self.order[k]] = (code, l)
                code += 1
                k += 1
            code <<= 1

    def segment_body(self, tc: int, th: int) -> bytes:
        return bytes([(tc << 4) | th]) + bytes(self.counts[1:]) + bytes(self.order)


def _category(v: int) -> int:
    return int(abs(v)).bit_length()


def _magnitude_bits(v: int, n: int) -> int:
    return v if v >= 0 else v + (1 << n) - 1


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value: int, n: int) -> None:
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self._byte(self.acc)
                self.acc, self.n = 0, 0

    def _byte(self, b: int) -> None:
        self.out.append(b)
        if b == 0xFF:
            self.out.append(0x00)  # byte stuffing

    def flush(self) -> None:
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)  # pad with one-bits


def encode(img: np.ndarray, *, sampling: tuple[int, int] = (1, 1), luma_q: np.ndarray | None = None,
           chroma_q: np.ndarray | None = None, restart: int = 0, q16: bool = False, one_dht: bool = True,
           app0: bool = True) -> tuple[bytes, np.ndarray]:
    """img: uint8 [H,W] (grey) or [H,W,3] (RGB).  sampling = (h, v) of the luma component
    (chroma is 1x1).  Returns (file bytes, the uint8 [H,W,3] a conforming reader decodes,
    with the IJG triangle-filter chroma upsampling and JFIF YCbCr -> RGB)."""
    grey = img.ndim == 2
    hgt, wid = img.shape[:2]
    hmax, vmax = (1, 1) if grey else sampling
    luma_q = quant_table(4, 0.3) if luma_q is None else luma_q
    chroma_q = quant_table(6, 0.4) if chroma_q is None else chroma_q
    mcux, mcuy = -(-wid // (8 * hmax)), -(-hgt // (8 * vmax))
    if grey:
        src = [img.astype(np.float64)]
        comps = [(1, 1, 1, 0)]  # (id, h, v, tq)
    else:
        ycc = rgb_to_ycbcr(img)
        src = [ycc[..., 0], ycc[..., 1], ycc[..., 2]]
        comps = [(1, hmax, vmax, 0), (2, 1, 1, 1), (3, 1, 1, 1)]
    qts = [luma_q, chroma_q]
    # component planes padded to whole MCUs; chroma is the box average of hmax x vmax pixels
    planes = []
    for (cid, h, v, tq), p in zip(comps, src):
        full = _pad_edge(p, mcuy * 8 * vmax, mcux * 8 * hmax)
        fy, fx = vmax // v, hmax // h
        planes.append(full.reshape(full.shape[0] // fy, fy, full.shape[1] // fx, fx).mean(axis=(1, 3)))
    # quantised coefficients per block, natural order
    coef = []
    for (cid, h, v, tq), p in zip(comps, planes):
        bh, bw = p.shape[0] // 8, p.shape[1] // 8
        blocks = (p - 128.0).reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
        f = np.einsum("xu,abxy,yv->abuv", BASIS, blocks, BASIS)  # F[u=row freq][v=col freq]
        coef.append(np.rint(f.reshape(bh, bw, 64) / qts[tq]).astype(np.int64))
    # symbol stream in MCU order, with DC prediction reset at each restart
    events = []  # (component index, block row, block col) in coding order
    for my in range(mcuy):
        for mx in range(mcux):
            for ci, (cid, h, v, tq) in enumerate(comps):
                for by in range(v):
                    for bx in range(h):
                        events.append((my * mcux + mx, ci, my * v + by, mx * h + bx))
    streams = []  # (starts a restart interval, table id, symbols)
    pred = [0] * len(comps)
    for idx, (mcu, ci, r, c) in enumerate(events):
        interval_start = bool(restart) and mcu > 0 and mcu % restart == 0 and events[idx - 1][0] != mcu
        if interval_start:
            pred = [0] * len(comps)
        blk = coef[ci][r, c][ZZ]
        diff = int(blk[0]) - pred[ci]
        pred[ci] = int(blk[0])
        syms = [("dc", _category(diff), diff)]
        run = 0
        last = max([k for k in range(1, 64) if blk[k] != 0], default=0)
        for k in range(1, last + 1):
            a = int(blk[k])
            if a == 0:
                run += 1
                continue
            while run > 15:
                syms.append(("ac", 0xF0, None))
                run -= 16
            syms.append(("ac", (run << 4) | _category(a), a))
            run = 0
        if last < 63:
            syms.append(("ac", 0x00, None))
        streams.append((interval_start, comps[ci][3], syms))
    tables = {}
    for kind in ("dc", "ac"):
        for t in (0, 1):
            freq: dict[int, int] = {}
            for _, tq, syms in streams:
                if tq != t:
                    continue
                for k, s, _ in syms:
                    if k == kind:
                        freq[s] = freq.get(s, 0) + 1
            if freq:
                tables[(kind, t)] = Huffman(freq)
    bw = _BitWriter()
    rst = 0
    for interval_start, tq, syms in streams:
        if interval_start:
            bw.flush()
            bw.out += bytes([0xFF, 0xD0 + rst % 8])
            rst += 1
        for kind, s, val in syms:
            code, l = tables[(kind, tq)].codes[s]
            bw.put(code, l)
            nbits = s if kind == "dc" else s & 15
            if val is not None and nbits:
                bw.put(_magnitude_bits(val, nbits), nbits)
    bw.flush()

    def seg(marker: int, body: bytes) -> bytes:
        return bytes([0xFF, marker]) + struct.pack(">H", len(body) + 2) + body

    out = b"\xff\xd8"
    if app0:
        out += seg(0xE0, b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00")
    out += seg(0xFE, b"test image")
    for t, q in enumerate(qts[: 1 if grey else 2]):
        body = bytes([(1 if q16 else 0) << 4 | t])
        body += b"".join(struct.pack(">H", int(q[z])) for z in ZZ) if q16 else bytes(int(q[z]) for z in ZZ)
        out += seg(0xDB, body)
    sof = struct.pack(">BHHB", 8, hgt, wid, len(comps)) + b"".join(bytes([cid, (h << 4) | v, tq])
                                                                      for cid, h, v, tq in comps)
    out += seg(0xC0, sof)
    dht = [tables[k].segment_body(0 if k[0] == "dc" else 1, k[1]) for k in sorted(tables)]
    out += seg(0xC4, b"".join(dht)) if one_dht else b"".join(seg(0xC4, d) for d in dht)
    if restart:
        out += seg(0xDD, struct.pack(">H", restart))
    sos = bytes([len(comps)]) + b"".join(bytes([cid, (tq << 4) | tq]) for cid, h, v, tq in comps) + b"\x00\x3f\x00"
    out += seg(0xDA, sos) + bytes(bw.out) + b"\xff\xd9"
    return out, expected_decode(coef, comps, qts, wid, hgt, hmax, vmax, grey)


def expected_decode(coef, comps, qts, wid, hgt, hmax, vmax, grey) -> np.ndarray:
    planes = []
    for (cid, h, v, tq), q in zip(comps, coef):
        bh, bw = q.shape[:2]
        f = (q * qts[tq]).reshape(bh, bw, 8, 8).astype(np.float64)
        pix = np.einsum("xu,abuv,yv->abxy", BASIS, f, BASIS) + 128.0
        pix = np.clip(np.floor(pix + 0.5), 0, 255)
        planes.append(pix.transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8))
    if grey:
        g = planes[0][:hgt, :wid].astype(np.uint8)
        return np.repeat(g[..., None], 3, axis=2)
    xs, ys = np.arange(wid), np.arange(hgt)
    full = []
    for (cid, h, v, tq), p in zip(comps, planes):
        fx, fy = hmax // h, vmax // v
        cw, ch = -(-wid * h // hmax), -(-hgt * v // vmax)
        i, j = xs // fx, ys // fy
        ni = np.clip(np.where(xs % 2 == 1, i + 1, i - 1), 0, cw - 1) if fx == 2 else i
        nj = np.clip(np.where(ys % 2 == 1, j + 1, j - 1), 0, ch - 1) if fy == 2 else j

        def col(ii):
            a = p[j[:, None], ii[None, :]]
            return 0.75 * a + 0.25 * p[nj[:, None], ii[None, :]] if fy == 2 else a

        full.append(0.75 * col(i) + 0.25 * col(ni) if fx == 2 else col(i))
    y, cb, cr = full[0], full[1] - 128.0, full[2] - 128.0
    rgb = np.stack([y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb], -1)
    return np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8)
