"""Minimal PNG reading / writing (zlib only): 8-bit greyscale, RGB, RGBA and palette-free
grey+alpha, non-interlaced, all five scanline filters.  Pixel values map to floats as
u8 / 255.0f, the conversion of backends/cuda/src/sad_cuda.cu:166-171.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def write_png(path: str, rgb_u8: np.ndarray) -> None:
    a = np.ascontiguousarray(rgb_u8, dtype=np.uint8)
    h, w = a.shape[:2]
    ch = 1 if a.ndim == 2 else a.shape[2]
    ctype = {1: 0, 3: 2, 4: 6}[ch]
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    png += _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def read_png(path: str) -> np.ndarray:
    """Returns uint8 [H,W,C] (C = 1, 2, 3 or 4)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if tag == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif tag == b"IDAT":
            idat.append(body)
        elif tag == b"IEND":
            break
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace != 0 or ctype == 3:
        raise ValueError(f"{path}: only 8-bit non-interlaced grey/RGB/RGBA PNGs are supported")
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), dtype=np.uint8)
    stride = w * ch
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        row = raw[y * (stride + 1):(y + 1) * (stride + 1)]
        ft, line = row[0], row[1:].astype(np.int32)
        cur = np.zeros(stride, dtype=np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        else:
            for i in range(stride):
                left = cur[i - ch] if i >= ch else 0
                up = prev[i]
                ul = prev[i - ch] if i >= ch else 0
                if ft == 1:
                    p = left
                elif ft == 3:
                    p = (left + up) >> 1
                else:
                    pa, pb, pc = abs(up - ul), abs(left - ul), abs(left + up - 2 * ul)
                    p = left if (pa <= pb and pa <= pc) else (up if pb <= pc else ul)
                cur[i] = (line[i] + p) & 0xFF
        out[y] = cur
        prev = cur
    return out.reshape(h, w, ch)


def load_image(path: str) -> np.ndarray:
    """PNG -> float32 [H,W,3] in [0,1] (grey is replicated, alpha dropped)."""
    a = read_png(path)
    if a.shape[2] in (1, 2):
        a = np.repeat(a[:, :, :1], 3, axis=2)
    a = a[:, :, :3]
    return a.astype(np.float32) / np.float32(255.0)


def save_image(path: str, rgb: np.ndarray) -> None:
    """float [H,W,3] in [0,1] -> 8-bit PNG."""
    write_png(path, np.clip(np.round(np.asarray(rgb) * 255.0), 0, 255).astype(np.uint8))
