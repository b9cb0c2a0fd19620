"""Tensor operators with the reference PyTorch extension's signatures
(backends/pytorch/torch_ext/cuda/sad_bindings.cu:496-1437), bound to `torch.ops.sad.*`.

The operators are implemented in C++ (sad_gb300/torch_ext/sad_torch_ops.cpp, loaded by
sad_gb300.torch_ops) on top of libsad_gb300's C ABI; each runs on the caller's current CUDA
stream and raises RuntimeError with the reference's argument messages.  Importing this
module registers them; it fails if another library already owns `torch.ops.sad`.
"""
from __future__ import annotations

import torch

from . import torch_ops

if not torch_ops.register():
    raise ImportError("torch.ops.sad is already registered by another library (the reference extension?); "
                      "sad_gb300.ops needs its own operators")

OP_NAMES = [
    "render_sad", "render_sad_padded", "init_candidates", "vpt_pass", "render_sad_backward",
    "clear_buffer", "pack_candidate_sites", "update_candidates_compact", "jfa_clear", "jfa_seed",
    "jfa_flood", "compute_gradients_tiled", "tau_diffuse", "adam_update",
    "compute_site_stats_tiled", "compute_densify_score_pairs", "compute_prune_score_pairs",
    "radix_sort_pairs", "write_split_indices", "split_sites", "prune_sites",
    "build_hilbert_pairs", "write_hilbert_order", "init_gradient_weighted",
]

_sad = torch.ops.sad


def __getattr__(name):
    """ops.<name> is torch.ops.sad.<name> for the operators of OP_NAMES."""
    if name in OP_NAMES:
        return getattr(_sad, name)
    raise AttributeError(name)


__all__ = list(OP_NAMES)
