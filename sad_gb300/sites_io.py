"""sites.txt / sites.json IO in the reference's format.

Text format (backends/cuda/src/sad_cuda.cu:277-338 read, 400-420 write): header lines
starting with '#' (one of them "# Image size: W H"), then one site per line with 10
floats in the order pos_x pos_y r g b log_tau radius dir_x dir_y log_aniso; 7-column lines
are accepted with dir = (1, 0), log_aniso = 0; other lines are skipped.  Written with 9
significant digits.  Returned arrays use the [N,10] device order
(pos, log_tau, radius, rgb, dir, log_aniso).
"""
from __future__ import annotations

import json
import os
import re

import numpy as np

# file column -> device column
_FILE_TO_DEV = [0, 1, 4, 5, 6, 2, 3, 7, 8, 9]


def load_sites(path: str):
    """Returns (sites [N,10] f32 device order, width or None, height or None)."""
    if os.path.splitext(path)[1].lower() == ".json":
        return load_sites_json(path)
    rows, w, h = [], None, None
    with open(path) as f:
        for line in f:
            t = line.strip()
            if not t:
                continue
            if t.startswith("#"):
                if "image size" in t.lower():
                    nums = re.findall(r"-?\d+", t)
                    if len(nums) >= 2:
                        w, h = int(nums[-2]), int(nums[-1])
                continue
            try:
                vals = [float(v) for v in t.split()]
            except ValueError:
                continue
            if len(vals) == 7:
                vals = vals + [1.0, 0.0, 0.0]
            if len(vals) != 10:
                continue
            dev = [0.0] * 10
            for fc, dc in enumerate(_FILE_TO_DEV):
                dev[dc] = vals[fc]
            rows.append(dev)
    if not rows:
        raise ValueError(f"No sites found in TXT: {path}")
    return np.asarray(rows, dtype=np.float32), w, h


def load_sites_json(path: str):
    """backends/cuda/src/sad_cuda.cu:340-390"""
    with open(path) as f:
        j = json.load(f)
    rows = []
    for s in j["sites"]:
        radius = s.get("radius", s.get("radius_sq", 0.0))
        d = s.get("aniso_dir", [1.0, 0.0])
        dx = d[0] if len(d) > 0 else 1.0
        dy = d[1] if len(d) > 1 else 0.0
        rows.append([s["pos"][0], s["pos"][1], s["log_tau"], radius, s["color"][0],
                     s["color"][1], s["color"][2], dx, dy, s.get("log_aniso", 0.0)])
    if not rows:
        raise ValueError(f"No sites found in JSON: {path}")
    return np.asarray(rows, dtype=np.float32), int(j["image_width"]), int(j["image_height"])


def save_sites(path: str, sites: np.ndarray, width: int, height: int) -> None:
    sites = np.asarray(sites, dtype=np.float32).reshape(-1, 10)
    with open(path, "w") as f:
        f.write("# SAD Sites (position_x, position_y, color_r, color_g, color_b, log_tau, radius, "
                "aniso_dir_x, aniso_dir_y, log_aniso)\n")
        f.write(f"# Image size: {width} {height}\n")
        f.write(f"# Total sites: {sites.shape[0]}\n")
        for s in sites:
            vals = [s[0], s[1], s[4], s[5], s[6], s[2], s[3], s[7], s[8], s[9]]
            f.write(" ".join(f"{float(np.float32(v)):.9g}" for v in vals) + "\n")
