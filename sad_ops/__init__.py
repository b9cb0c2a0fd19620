"""`sad_ops`, the Python package name of the reference's PyTorch extension
(backends/pytorch/torch_ext/sad_ops/__init__.py), backed by this library's C++ operators.

Importing it (or `sad_ops._sad_ext`, the module the reference's loader imports) registers
`torch.ops.sad.*` from libsad_torch_ops.so; the attributes mirror the reference package.
With this repository on the Python path, the reference's backends/pytorch modules run on
these operators unchanged.
"""
import torch

from . import _sad_ext  # noqa: F401  (registers torch.ops.sad)

ops = torch.ops.sad

render_sad = ops.render_sad
render_sad_padded = ops.render_sad_padded
render_sad_backward = ops.render_sad_backward
init_candidates = ops.init_candidates
vpt_pass = ops.vpt_pass

__all__ = [
    "ops",
    "render_sad",
    "render_sad_padded",
    "render_sad_backward",
    "init_candidates",
    "vpt_pass",
]
