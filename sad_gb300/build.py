"""Build libsad_gb300.so (all CUDA kernels + the C ABI) for sm_103a with nvcc.

    python -m sad_gb300.build [--force] [--verbose]

Translation units compile in parallel; the shared library and the sad_cuda command-line
host (sad_gb300/cli) land in sad_gb300/_lib/.
Nothing here needs a GPU (nvcc cross-compiles), and no torch headers are involved:
the boundary is the plain C ABI of include/sad_gb300.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_NAME = "libsad_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, "sad_gb300.h")]


def lib_path() -> str:
    return os.path.join(OUT_DIR, LIB_NAME)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    hdrs = headers()
    extra = list(extra_flags or [])
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs + [os.path.abspath(__file__)]):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", s, "-o", o]
            if s.endswith(".cpp"):
                cmd.insert(1, "-x")
                cmd.insert(2, "cu")
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    lib = lib_path()
    if jobs or not os.path.exists(lib):
        tmp = lib + ".tmp"
        run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, lib)
    build_cli(force=force, verbose=verbose)
    build_torch_ops(force=force, verbose=verbose)
    return lib


CLI_DIR = os.path.join(PKG, "cli")


def cli_path() -> str:
    return os.path.join(OUT_DIR, "sad_cuda")


def build_cli(force: bool = False, verbose: bool = False) -> str:
    """The sad_cuda-compatible command-line host (host C++ on the C ABI)."""
    srcs = sorted(os.path.join(CLI_DIR, f) for f in os.listdir(CLI_DIR) if f.endswith(".cpp"))
    deps = srcs + [os.path.join(CLI_DIR, f) for f in os.listdir(CLI_DIR) if f.endswith(".h")]
    deps += [os.path.join(INCLUDE, "sad_gb300.h"), lib_path(), os.path.abspath(__file__)]
    exe = cli_path()
    if not force and not _stale(exe, deps):
        return exe
    # no fused multiply-add contraction: the image decoders and resampling give the same
    # pixels on x86-64 and aarch64 hosts
    cmd = [nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CLI_DIR, *srcs,
           "-o", exe + ".tmp",
           "-L" + OUT_DIR, "-lsad_gb300", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(exe + ".tmp", exe)
    return exe


TORCH_EXT_DIR = os.path.join(PKG, "torch_ext")


def torch_ops_path() -> str:
    return os.path.join(OUT_DIR, "libsad_torch_ops.so")


def build_torch_ops(force: bool = False, verbose: bool = False) -> str | None:
    """The torch.ops.sad operator library (host C++ against torch's headers, on the C ABI).
    Skipped, returning None, when torch is not importable."""
    try:
        import torch
        from torch.utils import cpp_extension as ce
    except ImportError:
        return None
    src = os.path.join(TORCH_EXT_DIR, "sad_torch_ops.cpp")
    out = torch_ops_path()
    deps = [src, os.path.join(INCLUDE, "sad_gb300.h"), lib_path(), os.path.abspath(__file__), torch.__file__]
    if not force and not _stale(out, deps):
        return out
    try:
        incs = ce.include_paths(device_type="cuda")
        libs = ce.library_paths(device_type="cuda")
    except TypeError:  # older signature
        incs = ce.include_paths(cuda=True)
        libs = ce.library_paths(cuda=True)
    cuda_home = os.path.dirname(os.path.dirname(nvcc()))
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w",
           f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}",
           "-I" + INCLUDE, "-I" + os.path.join(cuda_home, "include"), *["-I" + i for i in incs],
           src, "-o", out + ".tmp", "-L" + OUT_DIR, "-lsad_gb300", *["-L" + d for d in libs],
           "-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu", "-ltorch_cuda",
           "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"torch operator build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
