"""ctypes binding of libsad_gb300.so (the C ABI declared in include/sad_gb300.h).

The library is loaded from sad_gb300/_lib/ (built by sad_gb300.build).  There is no
fallback: if the library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

c_u32p = C.POINTER(C.c_uint32)
c_f32p = C.POINTER(C.c_float)
vp = C.c_void_p
u32 = C.c_uint32
i32 = C.c_int
f32 = C.c_float
sz = C.c_size_t
st = C.c_int  # sad_status_t


class BppSolution(C.Structure):
    _fields_ = [("densify_percentile", f32), ("prune_percentile", f32),
                ("final_sites", i32), ("achieved_bpp", f32)]


class TrainConfig(C.Structure):
    _fields_ = [
        ("n_sites", i32), ("max_sites", i32), ("iterations", i32), ("target_bpp", f32),
        ("prune_percentile", f32), ("prune_during_densify", i32), ("prune_start", i32),
        ("prune_freq", i32), ("prune_end", i32), ("densify", i32), ("densify_start", i32),
        ("densify_freq", i32), ("densify_end", i32), ("densify_percentile", f32),
        ("densify_score_alpha", f32), ("cand_update_freq", i32), ("cand_update_passes", i32),
        ("cand_downscale", i32), ("cand_radius_scale", f32), ("cand_radius_probes", u32),
        ("cand_inject_count", u32), ("cand_hilbert_window", u32), ("cand_hilbert_probes", u32),
        ("lr_pos", f32), ("lr_tau", f32), ("lr_radius", f32), ("lr_color", f32), ("lr_dir", f32),
        ("lr_aniso", f32), ("lr_scale", f32), ("init_log_tau", f32), ("init_radius", f32),
        ("init_gradient_alpha", f32), ("beta1", f32), ("beta2", f32), ("eps", f32),
        ("ssim_weight", f32), ("log_freq", i32), ("use_graphs", i32),
        ("init_per_pixel", i32), ("autotune", i32),
    ]


class TrainerInfo(C.Structure):
    _fields_ = [("width", i32), ("height", i32), ("iteration", i32), ("site_buffer", i32),
                ("active_estimate", i32), ("capacity", i32), ("prune_percentile", f32),
                ("densify_percentile", f32), ("gpu_ms_gradients", C.c_double),
                ("gradient_launches", i32), ("kernel_launches", C.c_uint64),
                ("wide_far_refs", i32), ("tune_rounds", i32)]


class RenderConfig(C.Structure):
    _fields_ = [("candidate_passes", i32), ("use_jfa", i32), ("jfa_rounds", i32),
                ("cand_downscale", i32), ("cand_radius_scale", f32), ("cand_radius_probes", u32),
                ("cand_inject_count", u32), ("cand_hilbert_window", u32),
                ("cand_hilbert_probes", u32)]


class ExecutorConfig(C.Structure):
    _fields_ = [("workers", i32), ("hbm_budget_bytes", C.c_size_t), ("max_running_fits", i32)]


class RequestResult(C.Structure):
    _fields_ = [("status", i32), ("sites_written", i32), ("psnr", f32), ("queue_ms", C.c_double),
                ("run_ms", C.c_double), ("message", C.c_char * 192), ("iteration", i32)]


# name -> (restype, argtypes)
SIGNATURES = {
    "sad_last_error": (C.c_char_p, []),
    "sad_version": (C.c_char_p, []),
    "sad_abi_version": (i32, []),
    "sad_launch_count": (C.c_uint64, []),
    "sad_render": (st, [vp, vp, vp, vp, f32, u32, i32, i32, i32, i32, vp]),
    "sad_render_backward": (st, [vp, vp, vp, vp, vp, f32, u32, i32, i32, i32, i32, vp]),
    "sad_init_candidates": (st, [vp, vp, u32, u32, i32, i32, i32, vp]),
    "sad_clear_candidates": (st, [vp, vp, i32, i32, vp]),
    "sad_pack_candidate_sites": (st, [vp, vp, u32, vp]),
    "sad_jfa_seed": (st, [vp, vp, u32, i32, i32, i32, vp]),
    "sad_jfa_flood": (st, [vp, vp, vp, u32, u32, f32, i32, i32, i32, i32, i32, vp]),
    "sad_update_candidates": (st, [vp, vp, vp, vp, vp, u32, u32, f32, u32, f32, u32, u32, vp, vp,
                                   u32, u32, i32, i32, i32, i32, i32, vp]),
    "sad_jump_step_for_index": (u32, [u32, i32, i32]),
    "sad_pack_jump_step": (u32, [u32, i32, i32]),
    "sad_compute_gradients_tiled": (st, [vp, vp, vp, vp, vp] + [vp] * 10 +
                                    [vp, f32, u32, vp, u32, f32, i32, i32, i32, i32, vp]),
    "sad_compute_gradients_fixed_scratch_bytes": (sz, [u32, i32, i32]),
    "sad_compute_gradients_fixed": (st, [vp, vp, vp, vp, vp, vp, f32, u32, u32, f32, i32, i32, i32, i32,
                                         vp, vp, vp, sz, vp]),
    "sad_tau_diffuse": (st, [vp, vp, vp, vp, vp, vp, u32, f32, i32, i32, i32, vp]),
    "sad_adam_update": (st, [vp, vp] + [vp] * 10 + [f32] * 9 + [u32, u32, i32, i32, vp]),
    "sad_clear_gradients": (st, [vp] * 10 + [u32, vp]),
    "sad_clear_buffer": (st, [vp, u32, vp]),
    "sad_compute_densify_score_pairs": (st, [vp, vp, vp, vp, u32, f32, f32, u32, vp]),
    "sad_compute_prune_score_pairs": (st, [vp, vp, vp, u32, f32, u32, vp]),
    "sad_radix_sort_temp_bytes": (sz, [u32]),
    "sad_radix_sort_pairs": (st, [vp, u32, u32, vp, sz, vp]),
    "sad_radix_sort_pairs_noalloc": (st, [vp, u32, u32, vp]),
    "sad_write_split_indices": (st, [vp, vp, u32, vp]),
    "sad_prune_sites": (st, [vp, vp, u32, vp]),
    "sad_batch_create": (st, [C.POINTER(TrainConfig), i32, vp, vp, vp]),
    "sad_batch_destroy": (st, [vp]),
    "sad_batch_trainer": (st, [vp, i32, vp]),
    "sad_batch_init": (st, [vp]),
    "sad_batch_run": (st, [vp, i32]),
    "sad_batch_synchronize": (st, [vp]),
    "sad_batch_stream": (vp, [vp]),
    "sad_batch_enable_timing": (st, [vp, i32]),
    "sad_batch_gradient_ms": (st, [vp, vp]),
    "sad_compact_active_scratch_bytes": (sz, [u32]),
    "sad_compact_active": (st, [vp, u32, vp, vp, vp, sz, vp]),
    "sad_split_sites": (st, [vp, vp, vp, u32, vp, vp, vp, vp, vp, vp, vp, u32, vp, i32, i32, vp]),
    "sad_compute_site_stats": (st, [vp, vp, vp, vp, vp, f32, u32] + [vp] * 8 + [i32] * 4 + [vp]),
    "sad_init_temp_bytes": (sz, [u32]),
    "sad_init_gradient_weighted": (st, [vp, u32, vp, vp, f32, u32, f32, f32, i32, i32, vp, sz, vp]),
    "sad_hilbert_pairs": (st, [vp, vp, u32, u32, i32, i32, i32, vp]),
    "sad_write_hilbert_order": (st, [vp, vp, vp, u32, vp]),
    "sad_hilbert_bits_for_size": (i32, [i32, i32]),
    "sad_compute_mse": (st, [vp, vp, vp, vp, i32, i32, vp]),
    "sad_compute_ssim": (st, [vp, vp, vp, vp, i32, i32, vp]),
    "sad_count_active_sites": (st, [vp, vp, u32, vp]),
    "sad_solve_target_bpp": (st, [f32, i32, i32, i32, i32, i32, i32, i32, i32, i32, f32, i32, i32,
                                  i32, i32, f32, i32, C.POINTER(BppSolution)]),
    "sad_simulate_final_sites": (i32, [i32, i32, i32, i32, i32, i32, i32, f32, i32, i32, i32, i32,
                                       f32, i32]),
    "sad_train_config_default": (None, [C.POINTER(TrainConfig)]),
    "sad_trainer_create": (st, [C.POINTER(TrainConfig), i32, i32, C.POINTER(vp)]),
    "sad_trainer_destroy": (st, [vp]),
    "sad_trainer_memory_bytes": (sz, [C.POINTER(TrainConfig), i32, i32]),
    "sad_trainer_create_in": (st, [C.POINTER(TrainConfig), i32, i32, vp, sz, C.POINTER(vp)]),
    "sad_trainer_stream": (vp, [vp]),
    "sad_trainer_set_target_device": (st, [vp, vp, vp]),
    "sad_trainer_set_target_host": (st, [vp, vp, vp]),
    "sad_trainer_init": (st, [vp, vp, i32]),
    "sad_trainer_run": (st, [vp, i32]),
    "sad_trainer_render": (st, [vp, vp, C.POINTER(f32)]),
    "sad_trainer_get_sites": (st, [vp, vp, i32, i32, C.POINTER(i32)]),
    "sad_trainer_info": (st, [vp, C.POINTER(TrainerInfo)]),
    "sad_trainer_enable_timing": (st, [vp, i32]),
    "sad_trainer_fit_host": (st, [vp, vp, vp, vp, i32, C.POINTER(i32), C.POINTER(f32)]),
    "sad_render_config_default": (None, [C.POINTER(RenderConfig)]),
    "sad_render_scratch_bytes": (sz, [u32, i32, i32, i32]),
    "sad_render_from_sites": (st, [C.POINTER(RenderConfig), vp, u32, i32, i32, vp, vp, sz, vp]),
    "sad_render_from_sites_timed": (st, [C.POINTER(RenderConfig), vp, u32, i32, i32, vp, vp, sz, vp,
                                         C.POINTER(f32), C.POINTER(f32)]),
    "sad_pack_inference_sites": (st, [vp, u32, i32, i32, vp, vp, vp]),
    "sad_unpack_inference_sites": (st, [vp, vp, u32, i32, i32, vp, vp]),
    "sad_render_packed": (st, [vp, vp, vp, vp, vp, f32, u32, i32, i32, i32, i32, vp]),
    "sad_render_packed_scratch_bytes": (sz, [u32, i32, i32, i32]),
    "sad_render_packed_from_sites": (st, [C.POINTER(RenderConfig), vp, vp, u32, i32, i32, vp, vp, sz, vp]),
    "sad_trainer_render_packed": (st, [vp, vp, C.POINTER(f32), vp]),
    "sad_executor_config_default": (None, [C.POINTER(ExecutorConfig)]),
    "sad_executor_create": (st, [C.POINTER(ExecutorConfig), C.POINTER(vp)]),
    "sad_executor_submit_fit": (st, [vp, C.POINTER(TrainConfig), vp, vp, i32, i32, vp, i32,
                                     C.POINTER(RequestResult), C.POINTER(C.c_uint64)]),
    "sad_executor_submit_render": (st, [vp, C.POINTER(RenderConfig), vp, u32, i32, i32, vp,
                                        C.POINTER(RequestResult), C.POINTER(C.c_uint64)]),
    "sad_executor_open_fit": (st, [vp, C.POINTER(TrainConfig), vp, vp, i32, i32, vp, vp, vp]),
    "sad_executor_submit_continue": (st, [vp, C.c_uint64, i32, vp, i32, vp, vp]),
    "sad_executor_close_fit": (st, [vp, C.c_uint64, vp, vp]),
    "sad_executor_wait": (st, [vp, C.c_uint64]),
    "sad_executor_wait_all": (st, [vp]),
    "sad_executor_cancel": (st, [vp, C.c_uint64, C.POINTER(i32)]),
    "sad_executor_inject_slab_failures": (st, [vp, i32]),
    "sad_executor_destroy": (st, [vp]),
}

STATUS = {0: "SAD_OK", 1: "SAD_ERR_INVALID_ARGUMENT", 2: "SAD_ERR_CUDA", 3: "SAD_ERR_OUT_OF_MEMORY",
          4: "SAD_ERR_UNSUPPORTED", 5: "SAD_ERR_INTERNAL"}


class SadError(RuntimeError):
    """A libsad_gb300 call returned a non-OK status."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn}: {STATUS.get(code, code)}: {msg}")
        self.code = code


_LIB = None


def lib_path() -> str:
    return os.environ.get("SAD_GB300_LIB", _build.lib_path())


def load(build_if_missing: bool = False):
    """Load the shared library (optionally building it first)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                f"libsad_gb300.so not found at {path}; build it with `python -m sad_gb300.build`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def call(name: str, *args):
    """Call an entry point returning sad_status_t and raise SadError on failure."""
    lib = load()
    code = getattr(lib, name)(*args)
    if code != 0:
        msg = lib.sad_last_error().decode(errors="replace")
        raise SadError(name, code, msg)
    return code


def fn(name: str):
    return getattr(load(), name)
