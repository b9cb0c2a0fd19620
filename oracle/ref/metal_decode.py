"""Build the reference's packed-site decoder and packed render weights for the host: slice
the declarations up to decodePackedSite, voronoi_dmix2 and computePackedWeights out of
backends/metal/shaders/sad_common.metal (under the reference root given on the command
line) into oracle/_ref/metal_decode_slice.h, and compile them with metal_shim.h and
metal_decode_main.cpp into oracle/_ref/libref_metal_decode.so.  Needs the reference
checkout; nothing it writes is committed.

    python oracle/ref/metal_decode.py /path/to/reference
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(ROOT, "oracle", "_ref")
LIB = os.path.join(OUT, "libref_metal_decode.so")


def _function(lines: list[str], signature: str) -> tuple[int, int]:
    """Line span [first, last] of the function whose definition starts with `signature`."""
    first = next(i for i, l in enumerate(lines) if re.match(r"\s*" + re.escape(signature), l))
    last = next(i for i in range(first, len(lines)) if lines[i].rstrip() == "}")
    return first, last


def build(reference_root: str) -> str:
    src = os.path.join(reference_root, "backends", "metal", "shaders", "sad_common.metal")
    lines = open(src).read().splitlines()
    # the declarations up to decodePackedSite (types, constants, the unorm helpers), then
    # the distance and the packed render's softmax
    start = next(i for i, l in enumerate(lines) if l.strip() == "using namespace metal;") + 1
    spans = [(start, _function(lines, "inline VoronoiSite decodePackedSite(")[1]),
             _function(lines, "inline float voronoi_dmix2("),
             _function(lines, "inline bool computePackedWeights(")]
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(OUT, "metal_decode_slice.h"), "w") as f:
        for a, b in spans:
            f.write(f"// {src} lines {a + 1}-{b + 1}\n")
            f.write("\n".join(lines[a:b + 1]) + "\n")
    # no contraction: the slice is evaluated as written, in IEEE single precision
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", HERE, "-I", OUT,
                    os.path.join(HERE, "metal_decode_main.cpp"), "-o", LIB], check=True)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
