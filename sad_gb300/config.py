"""training_config.json handling (the reference's knob names and meaning).

Lookup order: $CONFIG_PATH, ./training_config.json, then the packaged default (the same
values as the reference's training_config.json).  Keys and defaults follow
backends/cuda/src/sad_cuda.cu:422-517 (Defaults / loadDefaults); the CLI-only options
(--lr, --ssim-weight, --log-freq, ...) are keyword overrides.
"""
from __future__ import annotations

import json
import os

from . import _lib

PACKAGED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "training_config.json")

# json key -> (TrainConfig field, type)
KEYS = {
    "DEFAULT_SITES": ("n_sites", int), "DEFAULT_MAX_SITES": ("max_sites", int),
    "DEFAULT_ITERS": ("iterations", int), "DEFAULT_TARGET_BPP": ("target_bpp", float),
    "PRUNE_PERCENTILE": ("prune_percentile", float),
    "PRUNE_DURING_DENSIFY": ("prune_during_densify", bool), "PRUNE_START": ("prune_start", int),
    "PRUNE_FREQ": ("prune_freq", int), "PRUNE_END": ("prune_end", int),
    "DENSIFY_START": ("densify_start", int), "DENSIFY_FREQ": ("densify_freq", int),
    "DENSIFY_END": ("densify_end", int), "DENSIFY_PERCENTILE": ("densify_percentile", float),
    "DENSIFY_SCORE_ALPHA": ("densify_score_alpha", float),
    "CAND_UPDATE_FREQ": ("cand_update_freq", int), "CAND_UPDATE_PASSES": ("cand_update_passes", int),
    "CAND_DOWNSCALE": ("cand_downscale", int), "CAND_RADIUS_SCALE": ("cand_radius_scale", float),
    "CAND_RADIUS_PROBES": ("cand_radius_probes", int), "CAND_INJECT_COUNT": ("cand_inject_count", int),
    "CAND_HILBERT_WINDOW": ("cand_hilbert_window", int),
    "CAND_HILBERT_PROBES": ("cand_hilbert_probes", int),
    "LR_POS_BASE": ("lr_pos", float), "LR_TAU_BASE": ("lr_tau", float),
    "LR_RADIUS_BASE": ("lr_radius", float), "LR_COLOR_BASE": ("lr_color", float),
    "LR_DIR_BASE": ("lr_dir", float), "LR_ANISO_BASE": ("lr_aniso", float),
    "INIT_LOG_TAU": ("init_log_tau", float), "INIT_RADIUS": ("init_radius", float),
    "BETA1": ("beta1", float), "BETA2": ("beta2", float), "EPS": ("eps", float),
}


def config_path() -> str:
    env = os.environ.get("CONFIG_PATH")
    if env:
        return env
    if os.path.exists("training_config.json"):
        return os.path.abspath("training_config.json")
    return PACKAGED


def load_json(path: str | None = None) -> dict:
    with open(path or config_path()) as f:
        return json.load(f)


def train_config(path: str | None = None, **overrides) -> _lib.TrainConfig:
    """TrainConfig from a training_config.json plus keyword overrides (field names)."""
    cfg = _lib.TrainConfig()
    _lib.load().sad_train_config_default(cfg)
    data = load_json(path)
    if "INIT_LOG_TAU" not in data or "INIT_RADIUS" not in data:
        raise ValueError("INIT_LOG_TAU and INIT_RADIUS must be set in training_config.json")
    for key, (field, typ) in KEYS.items():
        if key in data:
            setattr(cfg, field, int(bool(data[key])) if typ is bool else typ(data[key]))
    for field, value in overrides.items():
        if not hasattr(cfg, field):
            raise KeyError(f"unknown config field {field!r}")
        setattr(cfg, field, value)
    return cfg


def as_dict(cfg: _lib.TrainConfig) -> dict:
    return {name: getattr(cfg, name) for name, _ in cfg._fields_}
