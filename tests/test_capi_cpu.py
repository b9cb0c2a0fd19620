"""The C-ABI library without a GPU: it loads, exports every entry point the header
declares, validates arguments before touching the device, and its host-side schedule
functions agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "sad_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sad_[a-z0-9_]+)\s*\(", src)))


def test_library_loads_and_exports_every_declared_symbol(sadlib):
    names = header_functions()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(sadlib, n)]
    assert not missing, missing
    assert sadlib.sad_abi_version() == 1
    assert b"sm_103a" in sadlib.sad_version()


def test_binding_table_covers_the_header(sadlib):
    from sad_gb300 import _lib
    assert set(header_functions()) == set(_lib.SIGNATURES)


@pytest.mark.parametrize("w,h", [(1024, 1024), (640, 480), (7, 3)])
def test_jump_schedule_matches_oracle(sadlib, orc, w, h):
    for i in list(range(24)) + [65535, 65536, 70001]:
        assert sadlib.sad_jump_step_for_index(i, w, h) == orc.jump_step_for_index(i, w, h)
        assert sadlib.sad_pack_jump_step(i, w, h) == orc.pack_jump_step(i, w, h)


@pytest.mark.parametrize("bpp,w,h,n", [(1.0, 1024, 1024, 128000), (0.5, 512, 384, 20000),
                                       (2.0, 256, 256, 4096), (0.2, 777, 333, 50000)])
def test_bpp_rule_matches_oracle(sadlib, orc, bpp, w, h, n):
    from sad_gb300 import _lib
    args = (bpp, w, h, n, n, 4000, 1, 20, 3000, 20, 0.01, 1, 100, 3000, 40, 0.033, 65536)
    sol = _lib.BppSolution()
    _lib.call("sad_solve_target_bpp", *args, C.byref(sol))
    want = orc.solve_target_bpp(*args)
    assert sol.final_sites == int(want[2])
    assert np.float32(sol.prune_percentile) == want[1]
    assert np.float32(sol.densify_percentile) == want[0]


def test_hilbert_bits_match(sadlib, orc):
    for w, h in [(1, 1), (2, 2), (1024, 1024), (1025, 10), (12000, 9000)]:
        assert sadlib.sad_hilbert_bits_for_size(w, h) == orc.hilbert_bits_for_size(w, h)


def test_argument_errors_are_reported_without_a_device(sadlib):
    from sad_gb300 import _lib
    with pytest.raises(_lib.SadError, match="invalid image size"):
        _lib.call("sad_render", None, None, None, None, 1.0, 0, 0, 0, 1, 1, None)
    # beyond the kernels' 32-bit pixel offsets (3 * pixel): rejected, not overflowed
    big = 26755
    with pytest.raises(_lib.SadError, match="invalid image size"):
        _lib.call("sad_render", C.c_void_p(64), C.c_void_p(64), C.c_void_p(64), C.c_void_p(64), 1.0, 1,
                  big, big, 4, 4, None)
    assert sadlib.sad_compute_gradients_fixed_scratch_bytes(1000, big, big) == 0
    assert sadlib.sad_compute_gradients_fixed_scratch_bytes(1000, 26754, 26754) > 0
    cfg = _lib.TrainConfig()
    sadlib.sad_train_config_default(C.byref(cfg))
    assert sadlib.sad_trainer_memory_bytes(C.byref(cfg), big, big) == 0
    with pytest.raises(_lib.SadError, match="null buffer"):
        _lib.call("sad_render", None, None, None, None, 1.0, 0, 4, 4, 4, 4, None)
    with pytest.raises(_lib.SadError, match="temp smaller"):
        _lib.call("sad_radix_sort_pairs", C.c_void_p(64), 100, 0xFFFFFFFF, C.c_void_p(64), 8, None)
    with pytest.raises(_lib.SadError, match="must differ"):
        _lib.call("sad_jfa_flood", C.c_void_p(64), C.c_void_p(64), C.c_void_p(64), 1, 1, 1.0, 4, 4,
                  1, 4, 4, None)
    assert "must differ" in sadlib.sad_last_error().decode()


def test_scratch_queries_are_monotone(sadlib):
    f = sadlib.sad_radix_sort_temp_bytes
    assert f(1) <= f(1000) <= f(128000) <= f(1 << 20)
    assert f(128000) >= 128000 * 8
    r = sadlib.sad_render_scratch_bytes
    assert r(1000, 256, 256, 1) < r(1000, 1024, 1024, 1)
    assert r(1000, 1024, 1024, 2) < r(1000, 1024, 1024, 1)
    assert sadlib.sad_init_temp_bytes(128000) > 128000 * 4


def test_default_config_is_the_reference_training_config(sadlib):
    from sad_gb300 import _lib, config
    cfg = config.train_config()
    d = _lib.TrainConfig()
    sadlib.sad_train_config_default(d)
    for name, _ in d._fields_:
        assert getattr(cfg, name) == getattr(d, name), name
    assert (cfg.n_sites, cfg.iterations, cfg.cand_update_freq, cfg.cand_inject_count) == (128000, 4000, 8, 4)
    assert (cfg.cand_hilbert_window, cfg.cand_hilbert_probes) == (32, 1)


def test_torch_op_schemas_registered():
    """Every operator of the reference extension is registered with its exact schema."""
    import torch
    from sad_gb300 import torch_ops
    from torch_schemas import SCHEMAS
    assert torch_ops.register()
    assert len(SCHEMAS) == 24
    for name, schema in SCHEMAS.items():
        op = getattr(torch.ops.sad, name)
        assert str(op.default._schema) == "sad::" + schema, name


def test_sad_ops_package_mirrors_the_reference_extension():
    """`sad_ops` (the reference extension's package name) and the `sad_ops._sad_ext` module
    its loader imports register this library's operators."""
    import importlib

    import torch
    importlib.import_module("sad_ops._sad_ext")
    import sad_ops
    assert sad_ops.ops is torch.ops.sad
    for name in ("render_sad", "render_sad_padded", "render_sad_backward", "init_candidates", "vpt_pass"):
        assert getattr(sad_ops, name) is getattr(torch.ops.sad, name)
