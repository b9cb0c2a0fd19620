"""Tensor-level ops with the reference's torch.ops.sad interface, backed by libsad_gb300.

Each function mirrors one op of backends/pytorch/torch_ext/torch_binding.cpp:6-30 with the
argument checks and error messages of backends/pytorch/torch_ext/cuda/sad_bindings.cu
(RuntimeError on a failed check).  Two deliberate differences:
  * work is issued on the *current* CUDA stream (the reference always uses the default
    stream, which breaks CUDA-graph capture and stream overlap);
  * the adam tensor is read with the packed 20-float layout its [N,20] shape implies.
In-place ops return the (possibly contiguous-copied) tensor they wrote, as the
reference's do.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib

_I32 = torch.int32
_F32 = torch.float32
_F16 = torch.float16


def _check(cond: bool, msg: str) -> None:
    if not cond:
        raise RuntimeError(msg)


def _cuda(t: torch.Tensor, name: str) -> None:
    _check(isinstance(t, torch.Tensor) and t.is_cuda, f"{name} must be a CUDA tensor")


def _dtype(t: torch.Tensor, dt: torch.dtype, name: str) -> None:
    label = {torch.float32: "float32", torch.int32: "int32", torch.float16: "float16"}[dt]
    _check(t.dtype == dt, f"{name} must be {label}")


def _p(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(t: torch.Tensor):
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _cand(c: torch.Tensor, name: str) -> None:
    _cuda(c, name)
    _dtype(c, _I32, name)
    _check(c.dim() == 2 and c.size(1) == 4, f"{name} must be [M,4]")


def _sites(s: torch.Tensor, name: str = "sites") -> None:
    _cuda(s, name)
    _dtype(s, _F32, name)
    _check(s.dim() == 2 and s.size(1) == 10, f"{name} must be [N,10]")


def render_sad(cand0, cand1, sites, inv_scale_sq: float, width: int, height: int):
    """replaces sad_bindings.cu:496-538 (renderVoronoi)"""
    _cand(cand0, "cand0"); _cand(cand1, "cand1"); _sites(sites)
    _check(width > 0 and height > 0, "width/height must be positive")
    _check(cand0.size(0) == width * height, "cand0 size must match width*height")
    _check(cand1.size(0) == width * height, "cand1 size must match width*height")
    return render_sad_padded(cand0, cand1, sites, inv_scale_sq, width, height, width, height)


def render_sad_padded(cand0, cand1, sites, inv_scale_sq: float, width: int, height: int,
                      cand_width: int, cand_height: int):
    """replaces sad_bindings.cu:541-589 (renderVoronoiPadded)"""
    _cand(cand0, "cand0"); _cand(cand1, "cand1"); _sites(sites)
    _check(width > 0 and height > 0, "width/height must be positive")
    _check(cand_width > 0 and cand_height > 0, "invalid cand size")
    _check(cand0.size(0) == cand_width * cand_height, "cand0 size must match cand_width*cand_height")
    _check(cand1.size(0) == cand_width * cand_height, "cand1 size must match cand_width*cand_height")
    cand0, cand1, sites = cand0.contiguous(), cand1.contiguous(), sites.contiguous()
    out = torch.empty((height, width, 3), dtype=_F32, device=cand0.device)
    with torch.cuda.device(cand0.device):
        _lib.call("sad_render", _p(cand0), _p(cand1), _p(out), _p(sites), float(inv_scale_sq),
                  sites.size(0), width, height, cand_width, cand_height, _stream(cand0))
    return out


def init_candidates(width: int, height: int, site_count: int, seed: int):
    """replaces sad_bindings.cu:591-621; per-pixel neighbourhood mode when site_count == W*H"""
    _check(width > 0 and height > 0, "invalid cand size")
    _check(site_count >= 0, "site_count must be non-negative")
    dev = torch.device("cuda", torch.cuda.current_device())
    cand0 = torch.empty((width * height, 4), dtype=_I32, device=dev)
    cand1 = torch.empty_like(cand0)
    _lib.call("sad_init_candidates", _p(cand0), _p(cand1), site_count & 0xFFFFFFFF,
              seed & 0xFFFFFFFF, int(site_count == width * height), width, height, _stream(cand0))
    return cand0, cand1


def vpt_pass(cand0, cand1, sites, inv_scale_sq: float, width: int, height: int, jump: int,
             radius_probes: int, radius_scale: float, inject_count: int, seed: int):
    """replaces sad_bindings.cu:623-696 (vptPass): packs the sites to f16 and runs one pass
    with step = jump << 16 and no Hilbert probes; `seed` is unused, as in the reference."""
    del seed
    _cand(cand0, "cand0"); _cand(cand1, "cand1"); _sites(sites)
    _check(cand0.size(0) == width * height, "cand0 size must match width*height")
    _check(cand1.size(0) == width * height, "cand1 size must match width*height")
    cand0, cand1, sites = cand0.contiguous(), cand1.contiguous(), sites.contiguous()
    out0, out1 = torch.empty_like(cand0), torch.empty_like(cand1)
    packed = torch.empty((sites.size(0), 8), dtype=_F16, device=sites.device)
    s = _stream(cand0)
    with torch.cuda.device(cand0.device):
        _lib.call("sad_pack_candidate_sites", _p(sites), _p(packed), sites.size(0), s)
        _lib.call("sad_update_candidates", _p(cand0), _p(cand1), _p(out0), _p(out1), _p(packed),
                  sites.size(0), (jump << 16) & 0xFFFFFFFF, float(inv_scale_sq), 0,
                  float(radius_scale), radius_probes, inject_count, None, None, 0, 0, 1, width,
                  height, width, height, s)
    return out0, out1


def render_sad_backward(cand0, cand1, sites, grad_output, inv_scale_sq: float, width: int,
                        height: int):
    """replaces sad_bindings.cu:698-749 (renderVoronoiBackward): returns dL/dsites [N,10]"""
    _cand(cand0, "cand0"); _cand(cand1, "cand1"); _sites(sites)
    _cuda(grad_output, "grad_output"); _dtype(grad_output, _F32, "grad_output")
    _check(grad_output.dim() == 3 and grad_output.size(2) == 3, "grad_output must be [H,W,3]")
    _check(grad_output.size(0) == height and grad_output.size(1) == width,
           "grad_output size must match height/width")
    _check(cand0.size(0) == width * height, "cand0 size must match width*height")
    _check(cand1.size(0) == width * height, "cand1 size must match width*height")
    cand0, cand1 = cand0.contiguous(), cand1.contiguous()
    sites, grad_output = sites.contiguous(), grad_output.contiguous()
    grad_sites = torch.zeros((sites.size(0), 10), dtype=_F32, device=sites.device)
    with torch.cuda.device(cand0.device):
        _lib.call("sad_render_backward", _p(cand0), _p(cand1), _p(grad_output), _p(grad_sites),
                  _p(sites), float(inv_scale_sq), sites.size(0), width, height, width, height,
                  _stream(cand0))
    return grad_sites


def clear_buffer(buffer, count: int):
    """replaces sad_bindings.cu:751-764"""
    _cuda(buffer, "buffer"); _dtype(buffer, _F32, "buffer")
    buffer = buffer.contiguous()
    n = buffer.numel()
    if count <= 0 or count > n:
        count = n
    with torch.cuda.device(buffer.device):
        _lib.call("sad_clear_buffer", _p(buffer), count, _stream(buffer))
    return buffer


def pack_candidate_sites(sites, packed, site_count: int):
    """replaces sad_bindings.cu:766-784"""
    _sites(sites); _cuda(packed, "packed"); _dtype(packed, _F16, "packed")
    _check(packed.dim() == 2 and packed.size(1) == 8, "packed must be [N,8]")
    sites, packed = sites.contiguous(), packed.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    _check(site_count <= sites.size(0) and site_count <= packed.size(0), "site_count exceeds buffers")
    with torch.cuda.device(sites.device):
        _lib.call("sad_pack_candidate_sites", _p(sites), _p(packed), site_count, _stream(sites))
    return packed


def update_candidates_compact(cand0_in, cand1_in, cand0_out, cand1_out, packed_sites,
                              hilbert_order, hilbert_pos, inv_scale_sq: float, site_count: int,
                              step: int, step_high: int, radius_scale: float, radius_probes: int,
                              inject_count: int, hilbert_probes: int, hilbert_window: int,
                              cand_downscale: int, target_width: int, target_height: int,
                              cand_width: int, cand_height: int):
    """replaces sad_bindings.cu:786-863"""
    for t, nm in ((cand0_in, "cand0_in"), (cand1_in, "cand1_in"), (cand0_out, "cand0_out"),
                  (cand1_out, "cand1_out")):
        _cand(t, nm)
        _check(t.size(0) == cand_width * cand_height, f"{nm} size mismatch")
    _cuda(packed_sites, "packed_sites"); _dtype(packed_sites, _F16, "packed_sites")
    _check(packed_sites.dim() == 2 and packed_sites.size(1) == 8, "packed_sites must be [N,8]")
    cand0_in, cand1_in = cand0_in.contiguous(), cand1_in.contiguous()
    cand0_out, cand1_out = cand0_out.contiguous(), cand1_out.contiguous()
    packed_sites = packed_sites.contiguous()
    if site_count <= 0:
        site_count = packed_sites.size(0)
    ho = hp = None
    if hilbert_probes > 0 and hilbert_window > 0:
        _cuda(hilbert_order, "hilbert_order"); _cuda(hilbert_pos, "hilbert_pos")
        _dtype(hilbert_order, _I32, "hilbert_order"); _dtype(hilbert_pos, _I32, "hilbert_pos")
        ho, hp = hilbert_order.contiguous(), hilbert_pos.contiguous()
    with torch.cuda.device(cand0_in.device):
        _lib.call("sad_update_candidates", _p(cand0_in), _p(cand1_in), _p(cand0_out),
                  _p(cand1_out), _p(packed_sites), site_count, step & 0xFFFFFFFF,
                  float(inv_scale_sq), step_high & 0xFFFFFFFF, float(radius_scale), radius_probes,
                  inject_count, _p(ho), _p(hp), hilbert_probes, hilbert_window, cand_downscale,
                  target_width, target_height, cand_width, cand_height, _stream(cand0_in))
    return cand0_out


def jfa_clear(cand0, cand1, cand_width: int, cand_height: int):
    """replaces sad_bindings.cu:865-881"""
    _cand(cand0, "cand0"); _cand(cand1, "cand1")
    cand0, cand1 = cand0.contiguous(), cand1.contiguous()
    _check(cand0.size(0) >= cand_width * cand_height and cand1.size(0) >= cand_width * cand_height,
           "cand size must cover cand_width*cand_height")
    with torch.cuda.device(cand0.device):
        _lib.call("sad_clear_candidates", _p(cand0), _p(cand1), cand_width, cand_height,
                  _stream(cand0))
    return cand0


def jfa_seed(cand0, sites, site_count: int, cand_downscale: int, cand_width: int,
             cand_height: int):
    """replaces sad_bindings.cu:883-906 (lowest site id wins a shared texel)"""
    _cand(cand0, "cand0"); _sites(sites)
    _check(cand0.size(0) == cand_width * cand_height, "cand0 size must match cand_width*cand_height")
    cand0, sites = cand0.contiguous(), sites.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    with torch.cuda.device(cand0.device):
        _lib.call("sad_jfa_seed", _p(cand0), _p(sites), site_count, cand_width, cand_height,
                  cand_downscale, _stream(cand0))
    return cand0


def jfa_flood(cand0_in, cand0_out, sites, inv_scale_sq: float, site_count: int, step_size: int,
              cand_downscale: int, cand_width: int, cand_height: int):
    """replaces sad_bindings.cu:908-942"""
    _cand(cand0_in, "cand0_in"); _cand(cand0_out, "cand0_out"); _sites(sites)
    _check(cand0_in.size(0) == cand_width * cand_height, "cand0_in size must match cand_width*cand_height")
    _check(cand0_out.size(0) == cand_width * cand_height, "cand0_out size must match cand_width*cand_height")
    cand0_in, cand0_out, sites = cand0_in.contiguous(), cand0_out.contiguous(), sites.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    with torch.cuda.device(cand0_in.device):
        _lib.call("sad_jfa_flood", _p(cand0_in), _p(cand0_out), _p(sites), site_count, step_size,
                  float(inv_scale_sq), cand_width, cand_height, cand_downscale,
                  cand_width * cand_downscale, cand_height * cand_downscale, _stream(cand0_in))
    return cand0_out


def compute_gradients_tiled(cand0, cand1, target, rendered, mask, sites, grad_pos_x, grad_pos_y,
                            grad_log_tau, grad_radius, grad_color_r, grad_color_g, grad_color_b,
                            grad_dir_x, grad_dir_y, grad_log_aniso, removal_delta,
                            inv_scale_sq: float, site_count: int, compute_removal: int,
                            ssim_weight: float, cand_width: int, cand_height: int):
    """replaces sad_bindings.cu:944-1013 (grads and removal are accumulated)"""
    for t, nm in ((cand0, "cand0"), (cand1, "cand1")):
        _cuda(t, nm); _dtype(t, _I32, nm)
    for t, nm in ((target, "target"), (rendered, "rendered"), (mask, "mask"), (sites, "sites")):
        _cuda(t, nm); _dtype(t, _F32, nm)
    _check(target.dim() == 3 and target.size(2) == 3, "target must be [H,W,3]")
    _check(rendered.dim() == 3 and rendered.size(2) == 3, "rendered must be [H,W,3]")
    _check(mask.dim() == 2, "mask must be [H,W]")
    _check(mask.size(0) == target.size(0) and mask.size(1) == target.size(1), "mask size must match target")
    _check(sites.dim() == 2 and sites.size(1) == 10, "sites must be [N,10]")
    grads = [grad_pos_x, grad_pos_y, grad_log_tau, grad_radius, grad_color_r, grad_color_g,
             grad_color_b, grad_dir_x, grad_dir_y, grad_log_aniso]
    for g in grads + [removal_delta]:
        _cuda(g, "gradient buffer"); _dtype(g, _F32, "gradient buffer")
        _check(g.is_contiguous(), "gradient buffers must be contiguous")
    cand0, cand1 = cand0.contiguous(), cand1.contiguous()
    target, rendered = target.contiguous(), rendered.contiguous()
    mask, sites = mask.contiguous(), sites.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    h, w = target.size(0), target.size(1)
    with torch.cuda.device(cand0.device):
        _lib.call("sad_compute_gradients_tiled", _p(cand0), _p(cand1), _p(target), _p(rendered),
                  _p(mask), *[_p(g) for g in grads], _p(sites), float(inv_scale_sq), site_count,
                  _p(removal_delta), int(compute_removal), float(ssim_weight), w, h, cand_width,
                  cand_height, _stream(cand0))
    return grad_pos_x


def tau_diffuse(cand0, cand1, sites, grad_raw, grad_in, grad_out, site_count: int, lam: float,
                cand_downscale: int, cand_width: int, cand_height: int):
    """replaces sad_bindings.cu:1015-1057"""
    for t, nm in ((cand0, "cand0"), (cand1, "cand1")):
        _cuda(t, nm); _dtype(t, _I32, nm)
    _sites(sites)
    for t, nm in ((grad_raw, "grad_raw"), (grad_in, "grad_in"), (grad_out, "grad_out")):
        _cuda(t, nm); _dtype(t, _F32, nm)
    cand0, cand1, sites = cand0.contiguous(), cand1.contiguous(), sites.contiguous()
    grad_raw, grad_in, grad_out = grad_raw.contiguous(), grad_in.contiguous(), grad_out.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    with torch.cuda.device(cand0.device):
        _lib.call("sad_tau_diffuse", _p(cand0), _p(cand1), _p(sites), _p(grad_raw), _p(grad_in),
                  _p(grad_out), site_count, float(lam), cand_width, cand_height, cand_downscale,
                  _stream(cand0))
    return grad_out


def adam_update(sites, adam, grad_pos_x, grad_pos_y, grad_log_tau, grad_radius, grad_color_r,
                grad_color_g, grad_color_b, grad_dir_x, grad_dir_y, grad_log_aniso, lr_pos: float,
                lr_tau: float, lr_radius: float, lr_color: float, lr_dir: float,
                lr_aniso: float, beta1: float, beta2: float, eps: float, t: int, width: int,
                height: int):
    """replaces sad_bindings.cu:1059-1104 (every site of the tensor is stepped)"""
    _sites(sites); _cuda(adam, "adam"); _dtype(adam, _F32, "adam")
    _check(adam.dim() == 2 and adam.size(1) == 20, "adam must be [N,20]")
    _check(adam.size(0) >= sites.size(0), "adam must have a row per site")
    grads = [grad_pos_x, grad_pos_y, grad_log_tau, grad_radius, grad_color_r, grad_color_g,
             grad_color_b, grad_dir_x, grad_dir_y, grad_log_aniso]
    for g in grads:
        _cuda(g, "gradient buffer"); _dtype(g, _F32, "gradient buffer")
        _check(g.numel() >= sites.size(0), "gradient buffers must cover every site")
    sites, adam = sites.contiguous(), adam.contiguous()
    grads = [g.contiguous() for g in grads]
    with torch.cuda.device(sites.device):
        _lib.call("sad_adam_update", _p(sites), _p(adam), *[_p(g) for g in grads], float(lr_pos),
                  float(lr_tau), float(lr_radius), float(lr_color), float(lr_dir), float(lr_aniso),
                  float(beta1), float(beta2), float(eps), t, sites.size(0), width, height,
                  _stream(sites))
    return sites


def compute_site_stats_tiled(cand0, cand1, target, mask, sites, mass, energy, err_w, err_wx,
                             err_wy, err_wxx, err_wxy, err_wyy, inv_scale_sq: float,
                             site_count: int, cand_width: int, cand_height: int):
    """replaces sad_bindings.cu:1106-1161 (the 8 arrays are zeroed for site_count first,
    as launchComputeSiteStatsSimple does)"""
    for t, nm in ((cand0, "cand0"), (cand1, "cand1")):
        _cuda(t, nm); _dtype(t, _I32, nm)
    for t, nm in ((target, "target"), (mask, "mask"), (sites, "sites")):
        _cuda(t, nm); _dtype(t, _F32, nm)
    _check(target.dim() == 3 and target.size(2) == 3, "target must be [H,W,3]")
    _check(mask.dim() == 2, "mask must be [H,W]")
    _check(mask.size(0) == target.size(0) and mask.size(1) == target.size(1), "mask size must match target")
    _check(sites.dim() == 2 and sites.size(1) == 10, "sites must be [N,10]")
    outs = [mass, energy, err_w, err_wx, err_wy, err_wxx, err_wxy, err_wyy]
    for o in outs:
        _cuda(o, "stat buffer"); _dtype(o, _F32, "stat buffer")
        _check(o.is_contiguous(), "stat buffers must be contiguous")
    cand0, cand1 = cand0.contiguous(), cand1.contiguous()
    target, mask, sites = target.contiguous(), mask.contiguous(), sites.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    h, w = target.size(0), target.size(1)
    s = _stream(cand0)
    with torch.cuda.device(cand0.device):
        for o in outs:
            _lib.call("sad_clear_buffer", _p(o), site_count, s)
        _lib.call("sad_compute_site_stats", _p(cand0), _p(cand1), _p(target), _p(mask), _p(sites),
                  float(inv_scale_sq), site_count, *[_p(o) for o in outs], w, h, cand_width,
                  cand_height, s)
    return mass


def compute_densify_score_pairs(sites, mass, energy, pairs, site_count: int, min_mass: float,
                                score_alpha: float, pair_count: int):
    """replaces sad_bindings.cu:1163-1198"""
    _sites(sites)
    for t, nm in ((mass, "mass"), (energy, "energy")):
        _cuda(t, nm); _dtype(t, _F32, nm)
    _cuda(pairs, "pairs"); _dtype(pairs, _I32, "pairs")
    _check(pairs.dim() == 2 and pairs.size(1) == 2, "pairs must be [M,2]")
    sites, mass, energy, pairs = sites.contiguous(), mass.contiguous(), energy.contiguous(), pairs.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    if pair_count <= 0:
        pair_count = pairs.size(0)
    with torch.cuda.device(sites.device):
        _lib.call("sad_compute_densify_score_pairs", _p(sites), _p(mass), _p(energy), _p(pairs),
                  site_count, float(min_mass), float(score_alpha), pair_count, _stream(sites))
    return pairs


def compute_prune_score_pairs(sites, removal_delta, pairs, site_count: int, delta_norm: float,
                              pair_count: int):
    """replaces sad_bindings.cu:1200-1229"""
    _sites(sites)
    _cuda(removal_delta, "removal_delta"); _dtype(removal_delta, _F32, "removal_delta")
    _cuda(pairs, "pairs"); _dtype(pairs, _I32, "pairs")
    _check(pairs.dim() == 2 and pairs.size(1) == 2, "pairs must be [M,2]")
    sites, removal_delta, pairs = sites.contiguous(), removal_delta.contiguous(), pairs.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    if pair_count <= 0:
        pair_count = pairs.size(0)
    with torch.cuda.device(sites.device):
        _lib.call("sad_compute_prune_score_pairs", _p(sites), _p(removal_delta), _p(pairs),
                  site_count, float(delta_norm), pair_count, _stream(sites))
    return pairs


def radix_sort_pairs(pairs, max_key_exclusive: int):
    """replaces sad_bindings.cu:1231-1264"""
    _cuda(pairs, "pairs"); _dtype(pairs, _I32, "pairs")
    _check(pairs.dim() == 2 and pairs.size(1) == 2, "pairs must be [N,2]")
    pairs = pairs.contiguous()
    count = pairs.size(0)
    _check(count > 0, "pairs must be non-empty")
    nbytes = _lib.fn("sad_radix_sort_temp_bytes")(count)
    temp = torch.empty((nbytes + 15) // 16 * 16, dtype=torch.uint8, device=pairs.device)
    with torch.cuda.device(pairs.device):
        _lib.call("sad_radix_sort_pairs", _p(pairs), count, max_key_exclusive & 0xFFFFFFFF, _p(temp),
                  temp.numel(), _stream(pairs))
    return pairs


def write_split_indices(pairs, indices, num_to_split: int):
    """replaces sad_bindings.cu:1266-1282"""
    _cuda(pairs, "pairs"); _cuda(indices, "indices")
    _dtype(pairs, _I32, "pairs"); _dtype(indices, _I32, "indices")
    _check(pairs.dim() == 2 and pairs.size(1) == 2, "pairs must be [N,2]")
    _check(indices.dim() == 1, "indices must be [K]")
    _check(num_to_split <= indices.size(0) and num_to_split <= pairs.size(0), "num_to_split exceeds buffers")
    pairs, indices = pairs.contiguous(), indices.contiguous()
    with torch.cuda.device(pairs.device):
        _lib.call("sad_write_split_indices", _p(pairs), _p(indices), max(0, num_to_split), _stream(pairs))
    return indices


def split_sites(sites, adam, split_indices, mass, err_w, err_wx, err_wy, err_wxx, err_wxy,
                err_wyy, current_site_count: int, num_to_split: int, target):
    """replaces sad_bindings.cu:1284-1322"""
    _sites(sites); _cuda(adam, "adam"); _dtype(adam, _F32, "adam")
    _check(adam.dim() == 2 and adam.size(1) == 20, "adam must be [N,20]")
    _cuda(split_indices, "split_indices"); _dtype(split_indices, _I32, "split_indices")
    _cuda(target, "target"); _dtype(target, _F32, "target")
    _check(target.dim() == 3 and target.size(2) == 3, "target must be [H,W,3]")
    _check(current_site_count + num_to_split <= sites.size(0), "split children exceed the site buffer")
    sites, adam = sites.contiguous(), adam.contiguous()
    split_indices, target = split_indices.contiguous(), target.contiguous()
    stats = [t.contiguous() for t in (mass, err_w, err_wx, err_wy, err_wxx, err_wxy, err_wyy)]
    with torch.cuda.device(sites.device):
        _lib.call("sad_split_sites", _p(sites), _p(adam), _p(split_indices), num_to_split,
                  *[_p(t) for t in stats], current_site_count, _p(target), target.size(1),
                  target.size(0), _stream(sites))
    return sites


def prune_sites(sites, indices, count: int):
    """replaces sad_bindings.cu:1324-1339"""
    _sites(sites); _cuda(indices, "indices"); _dtype(indices, _I32, "indices")
    _check(count <= indices.numel(), "count exceeds indices")
    sites, indices = sites.contiguous(), indices.contiguous()
    with torch.cuda.device(sites.device):
        _lib.call("sad_prune_sites", _p(sites), _p(indices), max(0, count), _stream(sites))
    return sites


def build_hilbert_pairs(sites, pairs, site_count: int, padded_count: int, width: int, height: int,
                        bits: int):
    """replaces sad_bindings.cu:1341-1372"""
    _sites(sites); _cuda(pairs, "pairs"); _dtype(pairs, _I32, "pairs")
    _check(pairs.dim() == 2 and pairs.size(1) == 2, "pairs must be [M,2]")
    sites, pairs = sites.contiguous(), pairs.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    if padded_count <= 0:
        padded_count = pairs.size(0)
    else:
        _check(pairs.size(0) == padded_count, "pairs size must match padded_count")
    with torch.cuda.device(sites.device):
        _lib.call("sad_hilbert_pairs", _p(sites), _p(pairs), site_count, padded_count, width,
                  height, bits, _stream(sites))
    return pairs


def write_hilbert_order(pairs, order, pos, site_count: int):
    """replaces sad_bindings.cu:1374-1397"""
    for t, nm in ((pairs, "pairs"), (order, "order"), (pos, "pos")):
        _cuda(t, nm); _dtype(t, _I32, nm)
    _check(pairs.dim() == 2 and pairs.size(1) == 2, "pairs must be [N,2]")
    pairs, order, pos = pairs.contiguous(), order.contiguous(), pos.contiguous()
    if site_count <= 0:
        site_count = order.size(0)
    with torch.cuda.device(pairs.device):
        _lib.call("sad_write_hilbert_order", _p(pairs), _p(order), _p(pos), site_count, _stream(pairs))
    return order


def init_gradient_weighted(sites, target, mask, site_count: int, init_log_tau: float,
                           init_radius: float, gradient_alpha: float):
    """replaces sad_bindings.cu:1399-1437 (threshold 0.01 * alpha, 256 attempts per site;
    seeds handed out in site order)"""
    _sites(sites)
    for t, nm in ((target, "target"), (mask, "mask")):
        _cuda(t, nm); _dtype(t, _F32, nm)
    _check(target.dim() == 3 and target.size(2) == 3, "target must be [H,W,3]")
    _check(mask.dim() == 2, "mask must be [H,W]")
    _check(mask.size(0) == target.size(0) and mask.size(1) == target.size(1), "mask size must match target")
    sites, target, mask = sites.contiguous(), target.contiguous(), mask.contiguous()
    if site_count <= 0:
        site_count = sites.size(0)
    nbytes = _lib.fn("sad_init_temp_bytes")(site_count)
    temp = torch.empty(nbytes, dtype=torch.uint8, device=sites.device)
    with torch.cuda.device(sites.device):
        _lib.call("sad_init_gradient_weighted", _p(sites), site_count, _p(target), _p(mask),
                  0.01 * float(gradient_alpha), 256, float(init_log_tau), float(init_radius),
                  target.size(1), target.size(0), _p(temp), temp.numel(), _stream(sites))
    return sites


OP_NAMES = [
    "render_sad", "render_sad_padded", "init_candidates", "vpt_pass", "render_sad_backward",
    "clear_buffer", "pack_candidate_sites", "update_candidates_compact", "jfa_clear", "jfa_seed",
    "jfa_flood", "compute_gradients_tiled", "tau_diffuse", "adam_update",
    "compute_site_stats_tiled", "compute_densify_score_pairs", "compute_prune_score_pairs",
    "radix_sort_pairs", "write_split_indices", "split_sites", "prune_sites",
    "build_hilbert_pairs", "write_hilbert_order", "init_gradient_weighted",
]
