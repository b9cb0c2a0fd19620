"""Golden vectors of the 16-byte packed-site decode, made by the reference's own decoder.

The reference's packed serving format is packed by Swift (packed_inference.swift) and
decoded by a Metal function (backends/metal/shaders/sad_common.metal: decodePackedSite).
The decoder compiles as plain C++ under a shim of the Metal types (oracle/ref/metal_shim.h,
oracle/ref/metal_decode.py, built from the reference checkout).  This script packs seeded
site sets with the oracle's restatement of the packer, decodes the words with the
reference's decoder and writes tests/golden/packed_decode.npz: sites, words, quant,
width, height, decoded sites [n,10] and the decoder's active flags; and, for one small
image, the reference's packed render (computePackedWeights) of a candidate field.

    python tests/golden/make_packed_fixture.py /path/to/reference
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "oracle", "ref"), os.path.dirname(HERE)]

import orc  # noqa: E402
import metal_decode  # noqa: E402
from test_packed_format import random_sites  # noqa: E402


def reference_decode(lib, words, quant, w, h):
    n = words.shape[0]
    out = np.zeros((n, 10), np.float32)
    act = np.zeros(n, np.int32)
    f = lib.ref_decode_packed
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    words = np.ascontiguousarray(words, np.uint32)
    quant = np.ascontiguousarray(quant, np.float32)
    f(words.ctypes.data, quant.ctypes.data, n, w, h, out.ctypes.data, act.ctypes.data)
    return out, act


def reference_render(lib, words, quant, c0, c1, inv_s2, w, h):
    rgb = np.zeros((h, w, 3), np.float32)
    f = lib.ref_render_packed
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_int, C.c_void_p]
    words = np.ascontiguousarray(words, np.uint32)
    quant = np.ascontiguousarray(quant, np.float32)
    c0 = np.ascontiguousarray(c0, np.uint32)
    c1 = np.ascontiguousarray(c1, np.uint32)
    f(words.ctypes.data, quant.ctypes.data, words.shape[0], c0.ctypes.data, c1.ctypes.data, inv_s2, w, h,
      rgb.ctypes.data)
    return rgb


def main(reference_root: str) -> None:
    lib = C.CDLL(metal_decode.build(reference_root))
    cases = {}
    # random sets (unnormalised directions, colours past [0, 1], inactive sites) at two sizes
    for name, (n, w, h, seed) in {"a": (800, 300, 200, 3), "b": (500, 1024, 1024, 4)}.items():
        cases[name] = (random_sites(n, w, h, seed), w, h)
    # range ends and special words: every field at its minimum and maximum, axis directions,
    # log_aniso at +-4 and 0, a 1x1 image
    e = np.zeros((6, 10), np.float32)
    e[0] = [0, 0, 2.0, 1.0, 0.1, 0.2, 0.3, 1, 0, 0]
    e[1] = [299, 199, 6.0, 9.0, 0.9, 0.8, 0.7, -1, 0, 1.0]
    e[2] = [150, 100, 4.0, 5.0, 0.5, 0.5, 0.5, 0, 1, -4.0]
    e[3] = [10, 190, 3.0, 2.0, 0.2, 0.9, 0.4, 0, -1, 4.0]
    e[4] = [-1, -1, 100, 100, 5, 5, 5, 0, 1, 0]
    e[5] = [299, 0, 5.5, 8.5, 0.3, 0.3, 0.3, 0.6, 0.8, 0.5]
    cases["edges"] = (e, 300, 200)
    cases["one"] = (np.float32([[0.0, 0.0, 5.0, 4.0, 0.5, 0.5, 0.5, 1.0, 0.0, 0.0]]), 1, 1)
    out = {}
    for name, (sites, w, h) in cases.items():
        words, quant = orc.pack_inference_sites(sites, w, h)
        dec, act = reference_decode(lib, words, quant, w, h)
        out[f"{name}_sites"] = sites
        out[f"{name}_words"] = words
        out[f"{name}_quant"] = quant
        out[f"{name}_size"] = np.int32([w, h])
        out[f"{name}_decoded"] = dec
        out[f"{name}_active"] = act
    # the packed render (renderVoronoiPacked's softmax over the candidates) of a 64x48 image:
    # nearest-site candidate lists with an out-of-range id, a repeated id and an inactive
    # site among them
    import cases as scenes
    w, h, n = 64, 48, 200
    _, sites = scenes.scene(w, h, n, 5)
    sites[::7, 0:2] = -1.0
    words, quant = orc.pack_inference_sites(sites, w, h)
    c0, c1 = scenes.knn_field(sites, w, h)
    c1 = c1.copy()
    c1[::5, 3] = n + 7
    c1[1::5, 2] = c0[1::5, 0]
    inv_s2 = np.float32(1.0 / max(w, h) ** 2)
    out.update(render_words=words, render_quant=quant, render_c0=c0, render_c1=c1,
               render_size=np.int32([w, h]), render_inv_s2=np.float32([inv_s2]),
               render_rgb=reference_render(lib, words, quant, c0, c1, inv_s2, w, h))
    np.savez_compressed(os.path.join(HERE, "packed_decode.npz"), **out)
    print("wrote", os.path.join(HERE, "packed_decode.npz"), sorted(cases))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
