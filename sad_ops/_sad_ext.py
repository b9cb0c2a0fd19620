"""Stands in for the reference's compiled `sad_ops._sad_ext`: loads libsad_torch_ops.so,
which registers the `torch.ops.sad` schemas and their CUDA implementations."""
from sad_gb300 import torch_ops as _torch_ops

if not _torch_ops.register():
    raise ImportError("torch.ops.sad is already registered by another library")
