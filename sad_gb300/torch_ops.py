"""The reference's `torch.ops.sad` operators, registered from C++.

libsad_torch_ops.so (built from sad_gb300/torch_ext/sad_torch_ops.cpp by sad_gb300.build)
defines the schemas of backends/pytorch/torch_ext/torch_binding.cpp:6-30 verbatim and
implements every operator in C++ on libsad_gb300's C ABI, so code written against the
reference extension (`torch.ops.sad.render_sad(...)`) runs unchanged, with the host cost of
a C++ operator.  If another library already owns the `sad` namespace (the reference
extension itself), registration is refused and `register()` returns False.
"""
from __future__ import annotations

import os

import torch

LIBRARY_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libsad_torch_ops.so")
REGISTERED = False


def register() -> bool:
    """Load the operator library once per process; True when these operators own
    torch.ops.sad, False when another library registered the namespace first."""
    global REGISTERED
    if REGISTERED:
        return True
    if not os.path.exists(LIBRARY_PATH):
        from . import build
        build.build()
    if not os.path.exists(LIBRARY_PATH):
        raise RuntimeError(f"{LIBRARY_PATH} is missing (PyTorch was not importable at build time)")
    try:
        torch.ops.load_library(LIBRARY_PATH)
    except (RuntimeError, OSError) as e:
        if "sad" in str(e) and ("TORCH_LIBRARY" in str(e) or "namespace" in str(e)):
            return False
        raise
    REGISTERED = True
    return True
