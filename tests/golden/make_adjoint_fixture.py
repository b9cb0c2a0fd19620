"""Generate the golden fixture of the autograd adjoint from the reference's own kernel.

    oracle/ref/stage.sh /path/to/reference     # copy its sources to baseline/_ref/ (git-ignored)
    python tests/golden/make_adjoint_fixture.py [outdir]     # on a machine with a GPU

The reference's backward of its differentiable render is `render_sad_backward`
(backends/pytorch/torch_ext/cuda/sad_bindings.cu:100-207 for the kernel, :698-749 for the
operator: grad_sites [N,10] zero-initialised, one float atomicAdd per (pixel, candidate,
parameter)).  Its PyTorch extension is compiled from the staged sources with nvcc/g++
(oracle/ref/time_autograd.py: build_reference_ext) and loaded into a child process of its
own, so that no operator of this library is registered beside it.  Each case's inputs are
seeded (tests/cases.py) and are stored with the reference's output in
<outdir>/render_backward.npz (default: tests/golden/).

The cases cover a nearest-site field with inactive sites, a random field with empty slots,
ids >= n and duplicated ids, and a field with all-inactive lists (pixels that contribute
nothing), at non-multiple-of-16 sizes.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

CASES = {
    # name: (w, h, n, seed, field)
    "knn_64x48": (64, 48, 400, 50, "knn"),
    "random_61x37": (61, 37, 300, 51, "random"),
    "knn_97x65": (97, 65, 1200, 52, "knn"),
}


def make_inputs(path: str) -> None:
    sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
    import cases
    arrays = {}
    for name, (w, h, n, seed, field) in CASES.items():
        img, sites = cases.scene(w, h, n, seed)
        sites[::11, 0] = -1.0  # inactive sites
        if field == "knn":
            c0, c1 = cases.knn_field(sites, w, h)
        else:
            c0, c1 = cases.random_field(w, h, n, seed)
        # a band of pixels whose every candidate is inactive: no contribution
        dead = np.nonzero(sites[:, 0] < 0)[0].astype(np.uint32)
        rows = slice(0, w * 2)
        c0[rows] = dead[: 4]
        c1[rows] = dead[4: 8]
        gout = np.random.default_rng(seed).standard_normal((h, w, 3)).astype(np.float32)
        inv = np.float32(1.0 / max(w, h) ** 2)
        for k, v in (("cand0", c0), ("cand1", c1), ("sites", sites), ("grad_out", gout)):
            arrays[f"{name}_{k}"] = np.ascontiguousarray(v)
        arrays[f"{name}_params"] = np.array([w, h, n], np.int64)
        arrays[f"{name}_inv_s2"] = inv
    np.savez(path, **arrays)


def run_reference(inp: str, out: str) -> None:
    """Child process: the reference extension alone registers torch.ops.sad."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import time_autograd
    torch.ops.load_library(time_autograd.build_reference_ext())
    z = np.load(inp)
    res = {}
    for name in CASES:
        w, h, n = (int(v) for v in z[f"{name}_params"])
        c0 = torch.from_numpy(z[f"{name}_cand0"].view(np.int32)).cuda()
        c1 = torch.from_numpy(z[f"{name}_cand1"].view(np.int32)).cuda()
        s = torch.from_numpy(z[f"{name}_sites"]).cuda()
        g = torch.from_numpy(z[f"{name}_grad_out"]).cuda()
        inv = float(z[f"{name}_inv_s2"])
        res[f"{name}_render"] = torch.ops.sad.render_sad(c0, c1, s, inv, w, h).cpu().numpy()
        res[f"{name}_grad_sites"] = torch.ops.sad.render_sad_backward(c0, c1, s, g, inv, w, h).cpu().numpy()
    torch.cuda.synchronize()
    np.savez(out, **res)


def main(outdir: str) -> None:
    os.makedirs(outdir, exist_ok=True)
    tmp = tempfile.mkdtemp()
    inp, out = os.path.join(tmp, "in.npz"), os.path.join(tmp, "out.npz")
    make_inputs(inp)
    subprocess.run([sys.executable, os.path.abspath(__file__), "--child", inp, out], check=True)
    a, b = np.load(inp), np.load(out)
    arrays = {k: a[k] for k in a.files}
    arrays.update({k: b[k] for k in b.files})
    path = os.path.join(outdir, "render_backward.npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--child":
        run_reference(sys.argv[2], sys.argv[3])
    else:
        main(sys.argv[1] if len(sys.argv) > 1 else HERE)
