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
render_sad = _sad.render_sad
render_sad_padded = _sad.render_sad_padded
init_candidates = _sad.init_candidates
vpt_pass = _sad.vpt_pass
render_sad_backward = _sad.render_sad_backward
clear_buffer = _sad.clear_buffer
pack_candidate_sites = _sad.pack_candidate_sites
update_candidates_compact = _sad.update_candidates_compact
jfa_clear = _sad.jfa_clear
jfa_seed = _sad.jfa_seed
jfa_flood = _sad.jfa_flood
compute_gradients_tiled = _sad.compute_gradients_tiled
tau_diffuse = _sad.tau_diffuse
adam_update = _sad.adam_update
compute_site_stats_tiled = _sad.compute_site_stats_tiled
compute_densify_score_pairs = _sad.compute_densify_score_pairs
compute_prune_score_pairs = _sad.compute_prune_score_pairs
radix_sort_pairs = _sad.radix_sort_pairs
write_split_indices = _sad.write_split_indices
split_sites = _sad.split_sites
prune_sites = _sad.prune_sites
build_hilbert_pairs = _sad.build_hilbert_pairs
write_hilbert_order = _sad.write_hilbert_order
init_gradient_weighted = _sad.init_gradient_weighted
