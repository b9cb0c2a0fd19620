"""Seeded synthetic inputs standing in for the public image sets (Kodak, DIV2K, CLIC),
which are not available here.

Image: smooth 2-D linear gradient + Gaussian blobs (sigma ~ U[4,40] px, colours U[0,1]^3)
+ hard-edged random convex polygons, clamped to [0,1], float32 [H,W,3].  Blob / polygon
counts follow the benchmark definitions: 32 / 8 at 256^2 and 256 / 64 at 1024^2
(count = 32 (side/256)^1.5, polygons a quarter of that).
Sites: position U[0,W) x U[0,H) (+0.25 px so no site sits on a pixel centre), per-axis
log-scales N(0, 0.3), rotation U[0, pi); the det-1 metric keeps only the difference
(log_aniso = clamp(s2 - s1, -4, 4), dir = (cos t, sin t)); radius 4, log_tau 5, colour
sampled from the image at floor(position).
"""
from __future__ import annotations

import numpy as np


def synthetic_image(width: int, height: int, seed: int = 0, n_blobs: int | None = None,
                    n_polys: int | None = None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    side = float(np.sqrt(width * height))
    if n_blobs is None:
        n_blobs = max(1, int(round(32 * (side / 256.0) ** 1.5)))
    if n_polys is None:
        n_polys = max(1, n_blobs // 4)
    yy, xx = np.mgrid[0:height, 0:width].astype(np.float32)
    c0 = rng.uniform(0, 1, 3).astype(np.float32)
    c1 = rng.uniform(0, 1, 3).astype(np.float32)
    th = rng.uniform(0, 2 * np.pi)
    t = xx * np.cos(th) + yy * np.sin(th)
    t = (t - t.min()) / max(float(t.max() - t.min()), 1e-6)
    img = c0[None, None, :] + (c1 - c0)[None, None, :] * t[..., None]
    for _ in range(n_blobs):
        sig = rng.uniform(4, 40)
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        col = rng.uniform(0, 1, 3).astype(np.float32)
        r = int(3 * sig) + 1
        x0, x1 = max(0, int(cx) - r), min(width, int(cx) + r + 1)
        y0, y1 = max(0, int(cy) - r), min(height, int(cy) + r + 1)
        if x0 >= x1 or y0 >= y1:
            continue
        gx, gy = xx[y0:y1, x0:x1], yy[y0:y1, x0:x1]
        a = np.exp(-((gx - cx) ** 2 + (gy - cy) ** 2) / (2 * sig * sig))[..., None]
        img[y0:y1, x0:x1] += (col - img[y0:y1, x0:x1]) * a
    for _ in range(n_polys):
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        rad = rng.uniform(0.02, 0.08) * side
        k = int(rng.integers(3, 9))
        ang = np.sort(rng.uniform(0, 2 * np.pi, k))
        px, py = cx + rad * np.cos(ang), cy + rad * np.sin(ang)
        col = rng.uniform(0, 1, 3).astype(np.float32)
        x0, x1 = max(0, int(px.min())), min(width, int(px.max()) + 2)
        y0, y1 = max(0, int(py.min())), min(height, int(py.max()) + 2)
        if x0 >= x1 or y0 >= y1:
            continue
        gx, gy = xx[y0:y1, x0:x1], yy[y0:y1, x0:x1]
        inside = np.ones(gx.shape, dtype=bool)
        for i in range(k):  # convex: inside every edge half-plane (counter-clockwise)
            ax, ay, bx, by = px[i], py[i], px[(i + 1) % k], py[(i + 1) % k]
            inside &= (bx - ax) * (gy - ay) - (by - ay) * (gx - ax) >= 0
        img[y0:y1, x0:x1][inside] = col
    return np.clip(img, 0.0, 1.0).astype(np.float32)


def synthetic_sites(image: np.ndarray, n: int, seed: int = 0, log_tau: float = 5.0,
                    radius: float = 4.0) -> np.ndarray:
    h, w = image.shape[:2]
    rng = np.random.default_rng(seed + 1)
    px = np.floor(rng.uniform(0, w, n)) + 0.25
    py = np.floor(rng.uniform(0, h, n)) + 0.25
    px = np.minimum(px, w - 1 + 0.25)
    py = np.minimum(py, h - 1 + 0.25)
    s = rng.normal(0.0, 0.3, (n, 2))
    th = rng.uniform(0, np.pi, n)
    out = np.zeros((n, 10), dtype=np.float32)
    out[:, 0], out[:, 1] = px, py
    out[:, 2] = log_tau
    out[:, 3] = radius
    ix = np.clip(px.astype(np.int64), 0, w - 1)
    iy = np.clip(py.astype(np.int64), 0, h - 1)
    out[:, 4:7] = image[iy, ix]
    out[:, 7], out[:, 8] = np.cos(th), np.sin(th)
    out[:, 9] = np.clip(s[:, 1] - s[:, 0], -4.0, 4.0)
    return out


def quantize_u8(image: np.ndarray) -> np.ndarray:
    """The 8-bit image a PNG-reading caller would see, back in [0,1] float32."""
    u8 = np.round(np.clip(image, 0, 1) * 255.0).astype(np.float32)
    return u8 / np.float32(255.0)
