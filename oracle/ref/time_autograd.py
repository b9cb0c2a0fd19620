"""Time the autograd path, render_sad forward + render_sad_backward at 512x512 with 16,384
sites on one fixed candidate field: the reference's PyTorch extension (its
torch_ext/cuda/sad_bindings.cu and torch_binding.cpp with the CUDA backend's kernels, built
from the staged sources for sm_103a) against this library's torch.ops.sad.  Both register
the `sad` op namespace, so each runs in its own process; the field, sites and upstream
gradient are made once and shared through a file.  Prints one JSON line.

    oracle/ref/stage.sh /path/to/reference      (once, where the reference is present)
    python oracle/ref/time_autograd.py [--size 512] [--sites 16384] [--iters 200]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
STAGED = os.path.join(ROOT, "baseline", "_ref", "sad")


def build_reference_ext() -> str:
    """Compile the reference extension with nvcc / g++ directly (no cmake, no ninja) into
    baseline/_ref/torch_ext_build_<machine>/sad_reference_ext.so; reused while its sources
    are older."""
    import sysconfig

    import torch
    from torch.utils import cpp_extension as ce
    src = os.path.join(STAGED, "src")
    ext = os.path.join(STAGED, "torch_ext")
    import platform
    out_dir = os.path.join(ROOT, "baseline", "_ref", "torch_ext_build_" + platform.machine())
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "sad_reference_ext.so")
    kernels = ["render", "candidate_pack", "jfa", "gradients", "tau_diffusion", "adam", "densify_prune",
               "utils", "radix_sort"]
    cu = [os.path.join(ext, "cuda", "sad_bindings.cu")] + [os.path.join(src, k + ".cu") for k in kernels]
    cpp = [os.path.join(ext, "torch_binding.cpp")]
    if os.path.exists(so) and all(os.path.getmtime(f) < os.path.getmtime(so) for f in cu + cpp):
        return so
    try:
        incs = ce.include_paths(device_type="cuda")
    except TypeError:
        incs = ce.include_paths(cuda=True)
    incs = incs + [sysconfig.get_paths()["include"], src, ext]
    defs = ["-DCUDA_KERNEL", "-DTORCH_EXTENSION_NAME=sad_reference_ext", "-DTORCH_API_INCLUDE_EXTENSION_H",
            f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}"]
    inc = ["-I" + i for i in incs]
    jobs, objs = [], []
    for f in cu:
        o = os.path.join(out_dir, os.path.basename(f) + ".o")
        objs.append(o)
        jobs.append(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                     "--expt-relaxed-constexpr", "--extended-lambda", "-Xcompiler", "-fPIC", *defs, *inc,
                     "-c", f, "-o", o])
    for f in cpp:
        o = os.path.join(out_dir, os.path.basename(f) + ".o")
        objs.append(o)
        jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", *defs, *inc, "-c", f, "-o", o])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for j in jobs]
    for j, p in zip(jobs, procs):
        log = p.communicate()[0]
        if p.returncode != 0:
            raise RuntimeError(f"reference extension build failed: {' '.join(j)}\n{log[-4000:]}")
    try:
        libs = ["-L" + d for d in ce.library_paths(device_type="cuda")]
    except TypeError:
        libs = ["-L" + d for d in ce.library_paths(cuda=True)]
    link = ["g++", "-shared", "-o", so + ".tmp", *objs, *libs, "-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu",
            "-ltorch_cuda", "-L" + os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64"),
            "-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference extension link failed: {r.stdout}{r.stderr}")
    os.replace(so + ".tmp", so)
    return so


def load_reference_ops():
    """Registers the reference's torch.ops.sad.* in this process."""
    import torch
    torch.ops.load_library(build_reference_ext())


def make_case(path: str, size: int, n: int):
    """Synthetic sites and a candidate field built with this library's ops (seeded init,
    JFA seeds, 16 VPT passes); saved for both timing processes."""
    import torch
    sys.path.insert(0, ROOT)
    from sad_gb300 import torch_ops
    torch_ops.register()  # torch.ops.sad.* backed by this library
    from sad_gb300.synthetic import synthetic_image, synthetic_sites
    img = synthetic_image(size, size, seed=3)
    sites = torch.from_numpy(synthetic_sites(img, n, seed=3)).cuda()
    inv = 1.0 / (size * size)
    ops = torch.ops.sad
    c0, c1 = ops.init_candidates(size, size, n, 12345)
    ops.jfa_seed(c0, sites, n, 1, size, size)
    jump = 1
    while jump < size:
        jump *= 2
    for i in range(16):
        jump = max(1, jump // 2)
        c0, c1 = ops.vpt_pass(c0, c1, sites, inv, size, size, jump, 0, 64.0, 4, 1000 + i)
    grad = torch.from_numpy(np.random.default_rng(5).standard_normal((size, size, 3)).astype(np.float32))
    np.savez(path, c0=c0.cpu().numpy(), c1=c1.cpu().numpy(), sites=sites.cpu().numpy(), grad=grad.numpy(),
             inv=np.float32(inv), size=size)


def time_child(path: str, impl: str, iters: int, out: str):
    import torch
    if impl == "reference":
        load_reference_ops()
    else:
        sys.path.insert(0, ROOT)
        from sad_gb300 import torch_ops
        torch_ops.register()
    d = np.load(path)
    size = int(d["size"])
    inv = float(d["inv"])
    c0, c1 = torch.from_numpy(d["c0"]).cuda(), torch.from_numpy(d["c1"]).cuda()
    sites, grad = torch.from_numpy(d["sites"]).cuda(), torch.from_numpy(d["grad"]).cuda()
    ops = torch.ops.sad
    for _ in range(5):
        img = ops.render_sad(c0, c1, sites, inv, size, size)
        g = ops.render_sad_backward(c0, c1, sites, grad, inv, size, size)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd = bwd = 0.0
    for _ in range(iters):
        e[0].record(st)
        img = ops.render_sad(c0, c1, sites, inv, size, size)
        e[1].record(st)
        g = ops.render_sad_backward(c0, c1, sites, grad, inv, size, size)
        e[2].record(st)
        e[2].synchronize()
        fwd += e[0].elapsed_time(e[1])
        bwd += e[1].elapsed_time(e[2])
    np.savez(out, img=img.cpu().numpy(), g=g.cpu().numpy())
    print(json.dumps({"impl": impl, "fwd_ms": fwd / iters, "bwd_ms": bwd / iters}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--sites", type=int, default=16384)
    ap.add_argument("--iters", type=int, default=200)
    ap.add_argument("--child", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--case", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--out", default=None, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.child:
        time_child(args.case, args.child, args.iters, args.out)
        return
    d = tempfile.mkdtemp()
    case = os.path.join(d, "case.npz")
    subprocess.run([sys.executable, "-c", f"import sys; sys.path.insert(0, {HERE!r}); import time_autograd as t; "
                    f"t.make_case({case!r}, {args.size}, {args.sites})"], check=True)
    res = {}
    for impl in ("reference", "ours"):
        out = os.path.join(d, impl + ".npz")
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--child", impl, "--case", case, "--out", out,
                            "--iters", str(args.iters)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{impl} timing failed:\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}")
        res[impl] = json.loads(r.stdout.strip().splitlines()[-1])
        res[impl]["arrays"] = np.load(out)
    a, b = res["reference"]["arrays"], res["ours"]["arrays"]
    g_ref, g_ours = a["g"], b["g"]
    rel = float(np.linalg.norm(g_ours - g_ref) / max(np.linalg.norm(g_ref), 1e-30))
    out = {"workload": f"render_sad + render_sad_backward, {args.size}x{args.size}, {args.sites} sites, "
                       "one fixed candidate field (seeded init, JFA seeds, 16 VPT passes)",
           "iters": args.iters}
    for impl in ("reference", "ours"):
        out[impl] = {k: round(v, 4) for k, v in res[impl].items() if k.endswith("_ms")}
        out[impl]["fwd_bwd_ms"] = round(res[impl]["fwd_ms"] + res[impl]["bwd_ms"], 4)
    out["speedup_fwd_bwd"] = round(out["reference"]["fwd_bwd_ms"] / out["ours"]["fwd_bwd_ms"], 2)
    out["render_max_abs_diff"] = float(np.max(np.abs(a["img"] - b["img"])))
    out["grad_rel_l2_diff"] = rel
    print(json.dumps(out))


if __name__ == "__main__":
    main()
