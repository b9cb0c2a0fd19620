"""Autograd render and candidate updater with the reference's Python API.

Mirrors backends/pytorch/modules.py:11-134: SADRenderFunction saves only (sites, cand0,
cand1) and recomputes the softmax weights in backward; the candidate lists are
non-differentiable inputs.
"""
from __future__ import annotations

import torch

from . import ops


class SADRenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sites: torch.Tensor, cand0: torch.Tensor, cand1: torch.Tensor,
                inv_scale_sq: float, width: int, height: int) -> torch.Tensor:
        if sites.device.type != "cuda":
            raise RuntimeError("sites must be on CUDA")
        if sites.dtype != torch.float32:
            raise RuntimeError("sites must be float32")
        if cand0.dtype != torch.int32 or cand1.dtype != torch.int32:
            raise RuntimeError("candidates must be int32")
        if cand0.device != sites.device or cand1.device != sites.device:
            raise RuntimeError("candidates must be on the same device as sites")
        width, height, inv_scale_sq = int(width), int(height), float(inv_scale_sq)
        cand0, cand1, sites = cand0.contiguous(), cand1.contiguous(), sites.contiguous()
        out = ops.render_sad(cand0, cand1, sites, inv_scale_sq, width, height)
        ctx.save_for_backward(sites, cand0, cand1)
        ctx.inv_scale_sq, ctx.width, ctx.height = inv_scale_sq, width, height
        return out

    @staticmethod
    def backward(ctx, grad_output: torch.Tensor):
        sites, cand0, cand1 = ctx.saved_tensors
        if grad_output.device != sites.device:
            raise RuntimeError("grad_output must be on the same device as sites")
        grad_sites = ops.render_sad_backward(cand0, cand1, sites, grad_output.contiguous(),
                                             ctx.inv_scale_sq, ctx.width, ctx.height)
        return grad_sites, None, None, None, None, None


class SADRenderer(torch.nn.Module):
    def __init__(self, inv_scale_sq: float):
        super().__init__()
        self.inv_scale_sq = float(inv_scale_sq)

    def forward(self, sites, cand0, cand1, width: int, height: int, inv_scale_sq=None):
        inv = self.inv_scale_sq if inv_scale_sq is None else float(inv_scale_sq)
        return SADRenderFunction.apply(sites, cand0, cand1, inv, width, height)


class CandidateUpdater:
    """Random candidate init + VPT passes (backends/pytorch/modules.py:75-130)."""

    def __init__(self, width: int, height: int, site_count: int, seed: int = 1, device=None):
        self.width, self.height = int(width), int(height)
        self.site_count, self.seed = int(site_count), int(seed)
        if device is not None and not isinstance(device, torch.device):
            device = torch.device(device)
        if device is None:
            if not torch.cuda.is_available():
                raise RuntimeError("CUDA device required")
            device = torch.device("cuda")
        self.device = device
        self.reset()

    def reset(self, site_count=None, seed=None):
        if site_count is not None:
            self.site_count = int(site_count)
        if seed is not None:
            self.seed = int(seed)
        with torch.cuda.device(self.device):
            self.cand0, self.cand1 = ops.init_candidates(self.width, self.height, self.site_count,
                                                         self.seed)
        return self.cand0, self.cand1

    @torch.no_grad()
    def update(self, sites, inv_scale_sq: float, jump: int, radius_probes: int = 1,
               radius_scale: float = 1.0, inject_count: int = 0, seed=None):
        if seed is None:
            seed = self.seed
        if sites.device != self.cand0.device:
            raise RuntimeError("sites must be on the same device as candidates")
        self.cand0, self.cand1 = ops.vpt_pass(self.cand0, self.cand1, sites, float(inv_scale_sq),
                                              self.width, self.height, int(jump), int(radius_probes),
                                              float(radius_scale), int(inject_count), int(seed))
        return self.cand0, self.cand1

    def get(self):
        return self.cand0, self.cand1


__all__ = ["SADRenderFunction", "SADRenderer", "CandidateUpdater"]
