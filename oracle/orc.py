"""numpy front end of the CPU oracle (liboracle built from oracle/sad_oracle*.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs.  Every function returns numpy arrays; candidate fields are uint32
[W*H,4] pairs (cand0, cand1); sites are float32 [N,10] in device order.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_L = None
vp = C.c_void_p
u32, i32, f32, f64 = C.c_uint32, C.c_int, C.c_float, C.c_double


class FitConfig(C.Structure):
    _fields_ = [
        ("iterations", i32), ("n_sites", i32), ("max_sites", i32),
        ("prune_pct", f32), ("prune_start", i32), ("prune_freq", i32), ("prune_end", i32),
        ("densify", i32), ("densify_pct", f32), ("densify_alpha", f32), ("densify_start", i32),
        ("densify_freq", i32), ("densify_end", i32), ("prune_during_densify", i32),
        ("cand_freq", i32), ("cand_passes", i32), ("cand_radius_scale", f32),
        ("cand_radius_probes", u32), ("cand_inject", u32), ("hilbert_window", u32),
        ("hilbert_probes", u32), ("lr_pos", f32), ("lr_tau", f32), ("lr_radius", f32),
        ("lr_color", f32), ("lr_dir", f32), ("lr_aniso", f32), ("beta1", f32), ("beta2", f32),
        ("eps", f32), ("init_log_tau", f32), ("init_radius", f32), ("threads", i32),
    ]


def lib():
    global _L
    if _L is None:
        _L = C.CDLL(_build.build())
        _L.orc_f32_to_f16.restype = C.c_uint16
        _L.orc_f32_to_f16.argtypes = [f32]
        _L.orc_f16_to_f32.restype = f32
        _L.orc_f16_to_f32.argtypes = [C.c_uint16]
        for n in ("orc_jump_step_for_index", "orc_pack_jump_step"):
            getattr(_L, n).restype = u32
            getattr(_L, n).argtypes = [u32, i32, i32]
        _L.orc_hilbert_index.restype = u32
        _L.orc_hilbert_index.argtypes = [u32, u32, i32]
        _L.orc_hilbert_bits_for_size.restype = i32
        _L.orc_psnr.restype = f64
        _L.orc_ssim_sum.restype = f64
        _L.orc_count_active.restype = u32
        _L.orc_packed_distance.restype = f32
        _L.orc_packed_distance.argtypes = [vp, f32, f32, f32]
        _L.orc_simulate_final_sites.restype = i32
        _L.orc_simulate_final_sites.argtypes = [i32] * 7 + [f32] + [i32] * 4 + [f32, i32]
        _L.orc_solve_target_bpp.argtypes = [f32] + [i32] * 9 + [f32] + [i32] * 4 + [f32, i32, vp]
        _L.orc_fit_create.restype = vp
        _L.orc_fit_create.argtypes = [vp, vp, i32, i32, vp, i32]
        _L.orc_fit_run.argtypes = [vp, i32, i32]
        _L.orc_fit_psnr.restype = f64
        _L.orc_fit_psnr.argtypes = [vp]
        _L.orc_fit_sites.argtypes = [vp, vp, i32, i32]
        _L.orc_fit_destroy.argtypes = [vp]
        _L.orc_set_threads.argtypes = [i32]
    return _L


def _p(a: np.ndarray | None):
    return a.ctypes.data_as(vp) if a is not None else None


def _f(x) -> f32:
    return f32(float(x))


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def f32_to_f16_bits(x: float) -> int:
    return int(lib().orc_f32_to_f16(float(x)))


def jump_step_for_index(i, w, h):
    return int(lib().orc_jump_step_for_index(i, w, h))


def pack_jump_step(i, w, h):
    return int(lib().orc_pack_jump_step(i, w, h))


def hilbert_index(x, y, bits):
    return int(lib().orc_hilbert_index(x, y, bits))


def hilbert_bits_for_size(w, h):
    return int(lib().orc_hilbert_bits_for_size(i32(w), i32(h)))


def render(c0, c1, sites, w, h, cw=None, ch=None, inv_s2=None):
    cw, ch = cw or w, ch or h
    inv_s2 = inv_s2 if inv_s2 is not None else 1.0 / float(max(w, h)) ** 2
    c0, c1, sites = _c(c0, np.uint32), _c(c1, np.uint32), _c(sites, np.float32)
    out = np.zeros((h, w, 3), np.float32)
    lib().orc_render(_p(c0), _p(c1), _p(sites), u32(sites.shape[0]), i32(w), i32(h), i32(cw), i32(ch),
                     _f(inv_s2), _p(out))
    return out


def render_d(c0, c1, sites, w, h, inv_s2):
    c0, c1, sites = _c(c0, np.uint32), _c(c1, np.uint32), _c(sites, np.float64)
    out = np.zeros((h, w, 3), np.float64)
    lib().orc_render_d(_p(c0), _p(c1), _p(sites), u32(sites.shape[0]), i32(w), i32(h), f64(inv_s2), _p(out))
    return out


def render_backward(c0, c1, sites, grad_out, w, h, cw=None, ch=None, inv_s2=None):
    """Returns (grad [N,10] float64, abs_sum [N,10] float64)."""
    cw, ch = cw or w, ch or h
    inv_s2 = inv_s2 if inv_s2 is not None else 1.0 / float(max(w, h)) ** 2
    c0, c1, sites = _c(c0, np.uint32), _c(c1, np.uint32), _c(sites, np.float32)
    g = _c(grad_out, np.float32)
    n = sites.shape[0]
    grad, absg = np.zeros((n, 10)), np.zeros((n, 10))
    lib().orc_render_backward(_p(c0), _p(c1), _p(sites), u32(n), i32(w), i32(h), i32(cw), i32(ch),
                              _f(inv_s2), _p(g), _p(grad), _p(absg))
    return grad, absg


def render_backward_d(c0, c1, sites, grad_out, w, h, inv_s2):
    c0, c1, sites = _c(c0, np.uint32), _c(c1, np.uint32), _c(sites, np.float64)
    g = _c(grad_out, np.float64)
    grad = np.zeros((sites.shape[0], 10))
    lib().orc_render_backward_d(_p(c0), _p(c1), _p(sites), u32(sites.shape[0]), i32(w), i32(h),
                                f64(inv_s2), _p(g), _p(grad))
    return grad


def init_candidates(n, seed, per_pixel, w, h):
    c0 = np.zeros((w * h, 4), np.uint32)
    c1 = np.zeros((w * h, 4), np.uint32)
    lib().orc_init_candidates(_p(c0), _p(c1), u32(n), u32(seed), i32(per_pixel), i32(w), i32(h))
    return c0, c1


def pack_sites(sites):
    sites = _c(sites, np.float32)
    out = np.zeros((sites.shape[0], 8), np.uint16)
    lib().orc_pack_candidate_sites(_p(sites), _p(out), u32(sites.shape[0]))
    return out


def jfa_seed(c0, sites, w, h, ds=1):
    c0 = _c(c0, np.uint32).copy()
    sites = _c(sites, np.float32)
    lib().orc_jfa_seed(_p(c0), _p(sites), u32(sites.shape[0]), i32(w), i32(h), i32(ds))
    return c0


def jfa_flood(c0, sites, step, w, h, ds=1, tw=None, th=None, inv_s2=None):
    tw, th = tw or w * ds, th or h * ds
    inv_s2 = inv_s2 if inv_s2 is not None else 1.0 / float(max(tw, th)) ** 2
    c0, sites = _c(c0, np.uint32), _c(sites, np.float32)
    out = np.zeros_like(c0)
    lib().orc_jfa_flood(_p(c0), _p(out), _p(sites), u32(sites.shape[0]), u32(step), _f(inv_s2),
                        i32(w), i32(h), i32(ds), i32(tw), i32(th))
    return out


def vpt_pass(c0, c1, packed, n, step, step_high, w, h, radius_scale=64.0, radius_probes=0,
             inject=4, horder=None, hpos=None, hprobes=0, hwin=0, ds=1, tw=None, th=None,
             inv_s2=None):
    tw, th = tw or w * ds, th or h * ds
    inv_s2 = inv_s2 if inv_s2 is not None else 1.0 / float(max(tw, th)) ** 2
    c0, c1, packed = _c(c0, np.uint32), _c(c1, np.uint32), _c(packed, np.uint16)
    o0, o1 = np.zeros_like(c0), np.zeros_like(c1)
    ho = _c(horder, np.uint32) if horder is not None else None
    hp = _c(hpos, np.uint32) if hpos is not None else None
    lib().orc_vpt_pass(_p(c0), _p(c1), _p(o0), _p(o1), _p(packed), u32(n), u32(step), _f(inv_s2),
                       u32(step_high), _f(radius_scale), u32(radius_probes), u32(inject), _p(ho),
                       _p(hp), u32(hprobes), u32(hwin), i32(ds), i32(tw), i32(th), i32(w), i32(h))
    return o0, o1


def packed_distance(packed_row, ux, uy, inv_s2):
    r = _c(packed_row, np.uint16)
    return float(lib().orc_packed_distance(_p(r), float(ux), float(uy), float(inv_s2)))


def compute_gradients(c0, c1, target, sites, w, h, mask=None, rendered=None, ssim_weight=0.0,
                      removal=False, cw=None, ch=None, inv_s2=None):
    """Returns (grads [10,N] f64, abs [10,N] f64, removal [N] f64 or None)."""
    cw, ch = cw or w, ch or h
    inv_s2 = inv_s2 if inv_s2 is not None else 1.0 / float(max(w, h)) ** 2
    c0, c1, sites = _c(c0, np.uint32), _c(c1, np.uint32), _c(sites, np.float32)
    t = _c(target, np.float32)
    m = _c(mask, np.float32) if mask is not None else None
    r = _c(rendered, np.float32) if rendered is not None else None
    n = sites.shape[0]
    g, a = np.zeros((10, n)), np.zeros((10, n))
    rem = np.zeros(n) if removal else None
    lib().orc_compute_gradients(_p(c0), _p(c1), _p(t), _p(r), _p(m), _p(sites), u32(n), i32(w), i32(h),
                                i32(cw), i32(ch), _f(inv_s2), _f(ssim_weight), _p(g), _p(a), _p(rem))
    return g, a, rem


def compute_gradients_d(c0, c1, target, sites, w, h, mask=None):
    """FP64 form of compute_gradients' ten per-site sums for the MSE loss (no SSIM term):
    the render adjoint of dL/dpred = 2 (pred - target) on the pixels the mask keeps, with
    pred and every term in double.  Returns [10, N] float64."""
    inv_s2 = 1.0 / float(max(w, h)) ** 2
    s64 = np.asarray(sites, np.float64)
    gout = 2.0 * (render_d(c0, c1, s64, w, h, inv_s2) - np.asarray(target, np.float64))
    if mask is not None:
        gout *= (np.asarray(mask) > 0)[..., None]
    return render_backward_d(c0, c1, s64, gout, w, h, inv_s2).T


def tau_diffuse(c0, c1, sites, raw, gin, lam, w, h, ds=1):
    c0, c1, sites = _c(c0, np.uint32), _c(c1, np.uint32), _c(sites, np.float32)
    raw, gin = _c(raw, np.float32), _c(gin, np.float32)
    out = np.zeros_like(gin)
    lib().orc_tau_diffuse(_p(c0), _p(c1), _p(sites), _p(raw), _p(gin), _p(out), u32(sites.shape[0]),
                          _f(lam), i32(w), i32(h), i32(ds))
    return out


def adam_update(sites, adam, grads10, lr, beta1, beta2, eps, t, w, h):
    """grads10: [10,N] float32; lr: 6 learning rates.  Returns (sites, adam) copies."""
    s, a = _c(sites, np.float32).copy(), _c(adam, np.float32).copy()
    g = _c(grads10, np.float32)
    lib().orc_adam_update(_p(s), _p(a), _p(g), u32(s.shape[0]), *[_f(x) for x in lr], _f(beta1),
                          _f(beta2), _f(eps), u32(t), i32(w), i32(h))
    return s, a


def densify_pairs(sites, mass, energy, pair_count, min_mass, alpha):
    sites = _c(sites, np.float32)
    out = np.zeros((pair_count, 2), np.uint32)
    lib().orc_densify_score_pairs(_p(sites), _p(_c(mass, np.float32)), _p(_c(energy, np.float32)),
                                  _p(out), u32(sites.shape[0]), _f(min_mass), _f(alpha), u32(pair_count))
    return out


def prune_pairs(sites, removal, pair_count, delta_norm):
    sites = _c(sites, np.float32)
    out = np.zeros((pair_count, 2), np.uint32)
    lib().orc_prune_score_pairs(_p(sites), _p(_c(removal, np.float32)), _p(out), u32(sites.shape[0]),
                                _f(delta_norm), u32(pair_count))
    return out


def radix_sort_pairs(pairs, max_key_exclusive):
    p = _c(pairs, np.uint32).copy()
    lib().orc_radix_sort_pairs(_p(p), u32(p.shape[0]), u32(max_key_exclusive & 0xFFFFFFFF))
    return p


def prune_sites(sites, indices):
    s = _c(sites, np.float32).copy()
    idx = _c(indices, np.uint32)
    lib().orc_prune_sites(_p(s), _p(idx), u32(idx.shape[0]))
    return s


def split_sites(sites, adam, split_idx, stats7, cur, target, w, h):
    s, a = _c(sites, np.float32).copy(), _c(adam, np.float32).copy()
    idx = _c(split_idx, np.uint32)
    st = [_c(x, np.float32) for x in stats7]
    lib().orc_split_sites(_p(s), _p(a), _p(idx), u32(idx.shape[0]), *[_p(x) for x in st], u32(cur),
                          _p(_c(target, np.float32)), i32(w), i32(h))
    return s, a


def init_gradient_weighted(target, n, thr=0.01, max_attempts=256, init_log_tau=5.0,
                           init_radius=4.0, mask=None):
    h, w = target.shape[:2]
    s = np.zeros((n, 10), np.float32)
    lib().orc_init_gradient_weighted(_p(s), u32(n), _p(_c(target, np.float32)),
                                     _p(_c(mask, np.float32)) if mask is not None else None, _f(thr),
                                     u32(max_attempts), _f(init_log_tau), _f(init_radius), i32(w), i32(h))
    return s


def site_stats(c0, c1, target, sites, w, h, mask=None, cw=None, ch=None, inv_s2=None):
    cw, ch = cw or w, ch or h
    inv_s2 = inv_s2 if inv_s2 is not None else 1.0 / float(max(w, h)) ** 2
    sites = _c(sites, np.float32)
    n = sites.shape[0]
    st = np.zeros((8, n))
    lib().orc_site_stats(_p(_c(c0, np.uint32)), _p(_c(c1, np.uint32)), _p(_c(target, np.float32)),
                         _p(_c(mask, np.float32)) if mask is not None else None, _p(sites), u32(n),
                         i32(w), i32(h), i32(cw), i32(ch), _f(inv_s2), _p(st))
    return st


def hilbert_pairs(sites, padded, w, h, bits):
    sites = _c(sites, np.float32)
    out = np.zeros((padded, 2), np.uint32)
    lib().orc_hilbert_pairs(_p(sites), _p(out), u32(sites.shape[0]), u32(padded), i32(w), i32(h), i32(bits))
    return out


def hilbert_order(sorted_pairs, n):
    p = _c(sorted_pairs, np.uint32)
    order, pos = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    lib().orc_write_hilbert_order(_p(p), _p(order), _p(pos), u32(n))
    return order, pos


def psnr(rendered, target, mask=None):
    h, w = target.shape[:2]
    return float(lib().orc_psnr(_p(_c(rendered, np.float32)), _p(_c(target, np.float32)),
                                _p(_c(mask, np.float32)) if mask is not None else None, i32(w), i32(h)))


def ssim_sum(rendered, target, mask=None):
    h, w = target.shape[:2]
    return float(lib().orc_ssim_sum(_p(_c(rendered, np.float32)), _p(_c(target, np.float32)),
                                    _p(_c(mask, np.float32)) if mask is not None else None, i32(w), i32(h)))


def count_active(sites):
    s = _c(sites, np.float32)
    return int(lib().orc_count_active(_p(s), u32(s.shape[0])))


def simulate_final_sites(*args):
    return int(lib().orc_simulate_final_sites(*args))


def solve_target_bpp(*args):
    out = np.zeros(4, np.float32)
    lib().orc_solve_target_bpp(*args, _p(out))
    return out


class Fit:
    """CPU fit over the oracle kernels (the timed CPU baseline)."""

    def __init__(self, cfg: FitConfig, target: np.ndarray, init_sites: np.ndarray | None = None):
        self.target = _c(target, np.float32)
        h, w = self.target.shape[:2]
        self.cfg = cfg
        s = _c(init_sites, np.float32) if init_sites is not None else None
        self.h = lib().orc_fit_create(C.byref(cfg), _p(self.target), w, h, _p(s),
                                      s.shape[0] if s is not None else 0)

    def run(self, begin, end):
        lib().orc_fit_run(self.h, int(begin), int(end))

    def psnr(self):
        return float(lib().orc_fit_psnr(self.h))

    def sites(self, capacity, active_only=True):
        out = np.zeros((capacity, 10), np.float32)
        k = lib().orc_fit_sites(self.h, _p(out), capacity, int(active_only))
        return out[:k]

    def close(self):
        if self.h:
            lib().orc_fit_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def fit_config_from(train_cfg, threads=0) -> FitConfig:
    """Oracle fit config from a sad_gb300 TrainConfig (after the bpp rule is applied by the
    caller through prune_pct / densify_pct)."""
    c = FitConfig()
    c.iterations = train_cfg.iterations
    c.n_sites = train_cfg.n_sites
    c.max_sites = train_cfg.max_sites
    c.prune_pct = train_cfg.prune_percentile
    c.prune_start, c.prune_freq = train_cfg.prune_start, train_cfg.prune_freq
    c.prune_end = train_cfg.prune_end
    c.densify = train_cfg.densify
    c.densify_pct, c.densify_alpha = train_cfg.densify_percentile, train_cfg.densify_score_alpha
    c.densify_start, c.densify_freq, c.densify_end = (train_cfg.densify_start, train_cfg.densify_freq,
                                                      train_cfg.densify_end)
    c.prune_during_densify = train_cfg.prune_during_densify
    c.cand_freq, c.cand_passes = train_cfg.cand_update_freq, train_cfg.cand_update_passes
    c.cand_radius_scale = train_cfg.cand_radius_scale
    c.cand_radius_probes = train_cfg.cand_radius_probes
    c.cand_inject = train_cfg.cand_inject_count
    c.hilbert_window, c.hilbert_probes = train_cfg.cand_hilbert_window, train_cfg.cand_hilbert_probes
    s = train_cfg.lr_scale
    c.lr_pos, c.lr_tau, c.lr_radius = train_cfg.lr_pos * s, train_cfg.lr_tau * s, train_cfg.lr_radius * s
    c.lr_color, c.lr_dir, c.lr_aniso = train_cfg.lr_color * s, train_cfg.lr_dir * s, train_cfg.lr_aniso * s
    c.beta1, c.beta2, c.eps = train_cfg.beta1, train_cfg.beta2, train_cfg.eps
    c.init_log_tau, c.init_radius = train_cfg.init_log_tau, train_cfg.init_radius
    c.threads = threads
    return c


# training_config.json keys -> FitConfig fields, with the reference's defaults for keys a
# file leaves out (backends/cuda/src/sad_cuda.cu:422-517, loadDefaults; densify is on by
# default, sad_cuda.cu:609).  The learning-rate keys are the reference's *_BASE rates.
_JSON_KEYS = {
    "DEFAULT_SITES": ("n_sites", int, 128000), "DEFAULT_MAX_SITES": ("max_sites", int, 128000),
    "DEFAULT_ITERS": ("iterations", int, 4000), "PRUNE_PERCENTILE": ("prune_pct", float, 0.033),
    "PRUNE_DURING_DENSIFY": ("prune_during_densify", bool, True), "PRUNE_START": ("prune_start", int, 100),
    "PRUNE_FREQ": ("prune_freq", int, 40), "PRUNE_END": ("prune_end", int, 3000),
    "DENSIFY_START": ("densify_start", int, 20), "DENSIFY_FREQ": ("densify_freq", int, 20),
    "DENSIFY_END": ("densify_end", int, 3000), "DENSIFY_PERCENTILE": ("densify_pct", float, 0.01),
    "DENSIFY_SCORE_ALPHA": ("densify_alpha", float, 0.7), "CAND_UPDATE_FREQ": ("cand_freq", int, 8),
    "CAND_UPDATE_PASSES": ("cand_passes", int, 1), "CAND_RADIUS_SCALE": ("cand_radius_scale", float, 64.0),
    "CAND_RADIUS_PROBES": ("cand_radius_probes", int, 0), "CAND_INJECT_COUNT": ("cand_inject", int, 4),
    "CAND_HILBERT_WINDOW": ("hilbert_window", int, 32), "CAND_HILBERT_PROBES": ("hilbert_probes", int, 1),
    "LR_POS_BASE": ("lr_pos", float, 0.025), "LR_TAU_BASE": ("lr_tau", float, 0.01),
    "LR_RADIUS_BASE": ("lr_radius", float, 0.01), "LR_COLOR_BASE": ("lr_color", float, 0.01),
    "LR_DIR_BASE": ("lr_dir", float, 0.0025), "LR_ANISO_BASE": ("lr_aniso", float, 0.025),
    "INIT_LOG_TAU": ("init_log_tau", float, 5.0), "INIT_RADIUS": ("init_radius", float, 4.0),
    "BETA1": ("beta1", float, 0.9), "BETA2": ("beta2", float, 0.999), "EPS": ("eps", float, 1e-8),
}


def fit_config_json(path: str, w: int, h: int, target_bpp: float | None = 1.0, threads: int = 0,
                    **overrides) -> FitConfig:
    """Oracle fit config read straight from a training_config.json (no product code
    involved), with the bpp rule applied when target_bpp > 0: the densify / prune
    percentiles are scaled as solveTargetBpp does (backends/cuda/src/sad_cuda.cu:904-1066,
    max split 65536 per event, sad_cuda.cu:1095)."""
    import json
    with open(path) as f:
        data = json.load(f)
    c = FitConfig()
    c.densify = 1
    for key, (field, typ, default) in _JSON_KEYS.items():
        v = data.get(key, default)
        setattr(c, field, int(bool(v)) if typ is bool else typ(v))
    for field, v in overrides.items():
        setattr(c, field, v)
    if target_bpp and target_bpp > 0:
        sol = solve_target_bpp(float(target_bpp), int(w), int(h), c.n_sites, c.max_sites, c.iterations,
                               c.densify, c.densify_start, c.densify_end, c.densify_freq, c.densify_pct,
                               c.prune_during_densify, c.prune_start, c.prune_end, c.prune_freq,
                               c.prune_pct, 65536)
        c.densify_pct, c.prune_pct = float(sol[0]), float(sol[1])
    c.threads = int(threads)
    return c


def timed_fit_sample(cfg: FitConfig, target: np.ndarray, first: int, chunks: list[int]):
    """Bounded CPU sample of one fit: iterations [0, first) run untimed (setup), then each
    chunk of consecutive iterations is timed on its own.  Returns the per-chunk seconds."""
    import time
    f = Fit(cfg, target)
    try:
        f.run(0, first)
        it, out = first, []
        for k in chunks:
            t0 = time.perf_counter()
            f.run(it, it + k)
            out.append(time.perf_counter() - t0)
            it += k
        return out
    finally:
        f.close()


def pack_inference_sites(sites, w, h):
    """16-byte quantised sites: (packed [N,4] u32, quant [10] f32)."""
    sites = _c(sites, np.float32)
    n = sites.shape[0]
    packed = np.zeros((n, 4), np.uint32)
    quant = np.zeros(10, np.float32)
    lib().orc_pack_inference_sites(_p(sites), u32(n), i32(w), i32(h), _p(packed), _p(quant))
    return packed, quant


def unpack_inference_sites(packed, quant, w, h):
    packed = _c(packed, np.uint32)
    quant = _c(quant, np.float32)
    out = np.zeros((packed.shape[0], 10), np.float32)
    lib().orc_unpack_inference_sites(_p(packed), _p(quant), u32(packed.shape[0]), i32(w), i32(h), _p(out))
    return out
