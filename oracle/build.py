"""Build the CPU oracle (test infrastructure) with gcc.

    python oracle/build.py            -> oracle/_build/libsad_oracle.so

-ffp-contract=off keeps the arithmetic identical on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsad_oracle.so")
SOURCES = ["sad_oracle.c", "sad_oracle_fit.c"]


def build(force=False, verbose=False):
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "sad_oracle.h")]
    if not force and os.path.exists(LIB):
        lib_m = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_m for s in srcs):
            return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-strict-aliasing", "-Wall", "-Wno-unused-function",
           *[os.path.join(HERE, s) for s in SOURCES], "-o", LIB + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
