"""The sad_cuda-compatible command-line host without a GPU: its PNG codec (sad_gb300/cli/png.cpp,
driven through tests/cli/png_check.cpp) against PNGs encoded here with zlib over every colour
type, bit depth and scanline filter the decoder accepts; its baseline JPEG reader
(sad_gb300/cli/jpeg.cpp; the reference host reads JPEG through stb_image,
backends/cuda/src/sad_cuda.cu:141) against files from tests/jpeg_encode.py; and the argument / configuration
handling whose exit codes follow backends/cuda/src/sad_cuda.cu:459-517 (missing
training_config.json or INIT_* keys -> exit 1) and :754-895 (--help -> 0, unknown flag -> 1).
"""
import json
import os
import shutil
import struct
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI_SRC = os.path.join(ROOT, "sad_gb300", "cli")
PACKAGED_CONFIG = os.path.join(ROOT, "sad_gb300", "training_config.json")


# ---------------------------------------------------------------------------
# PNG encoder for the test inputs (RFC 2083 scanline filters, zlib at several levels)
# ---------------------------------------------------------------------------
def _chunk(tag, data):
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _pack_row(samples, depth):
    """samples: 1-D int array of one row (channels interleaved) -> packed bytes."""
    if depth == 16:
        return b"".join(struct.pack(">H", int(v)) for v in samples)
    if depth == 8:
        return bytes(int(v) for v in samples)
    per = 8 // depth
    out = bytearray((len(samples) + per - 1) // per)
    for i, v in enumerate(samples):
        out[i // per] |= int(v) << (8 - depth * (i % per + 1))
    return bytes(out)


def _filter_row(row, prev, bpp, ftype):
    out = bytearray(len(row))
    for i in range(len(row)):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        pred = (0, a, b, (a + b) // 2, _paeth(a, b, c))[ftype]
        out[i] = (row[i] - pred) & 0xFF
    return bytes([ftype]) + bytes(out)


def encode_png(samples, ctype, depth, rng, level=6, palette=None, split_idat=False):
    h, w, chans = samples.shape
    rows, prev = [], bytes(((w * chans * depth) + 7) // 8)
    bpp = max(1, chans * depth // 8)
    for y in range(h):
        row = _pack_row(samples[y].reshape(-1), depth)
        rows.append(_filter_row(row, prev, bpp, int(rng.integers(0, 5))))
        prev = row
    z = zlib.compress(b"".join(rows), level)
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        png += _chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    png += _chunk(b"tEXt", b"Comment\x00ancillary chunk")
    if split_idat:
        k = len(z) // 3 + 1
        for i in range(0, len(z), k):
            png += _chunk(b"IDAT", z[i:i + k])
    else:
        png += _chunk(b"IDAT", z)
    return png + _chunk(b"IEND", b"")


def expected_rgb(samples, ctype, depth, palette=None):
    s = samples.astype(np.int64)
    if ctype == 3:
        return palette[s[..., 0]].astype(np.uint8)
    if depth == 16:
        s = s >> 8
    elif depth < 8:
        s = s * 255 // ((1 << depth) - 1)
    if ctype in (0, 4):
        return np.repeat(s[..., :1], 3, axis=2).astype(np.uint8)
    return s[..., :3].astype(np.uint8)


@pytest.fixture(scope="module")
def png_check(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("png") / "png_check")
    subprocess.run([cxx, "-O1", "-std=c++17", "-ffp-contract=off", "-I" + CLI_SRC, os.path.join(ROOT, "tests", "cli", "png_check.cpp"),
                    os.path.join(CLI_SRC, "png.cpp"), os.path.join(CLI_SRC, "jpeg.cpp"), "-o", exe], check=True)
    return exe


def _read(png_check, path, tmp_path):
    raw = tmp_path / "out.raw"
    r = subprocess.run([png_check, "read", str(path), str(raw)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    data = raw.read_bytes()
    head, body = data.split(b"\n", 1)
    w, h, gray = (int(v) for v in head.split())
    return np.frombuffer(body, np.uint8).reshape(h, w, 3), bool(gray)


CASES = [  # (colour type, bit depth)
    (0, 1), (0, 2), (0, 4), (0, 8), (0, 16),
    (2, 8), (2, 16),
    (3, 1), (3, 2), (3, 4), (3, 8),
    (4, 8), (4, 16),
    (6, 8), (6, 16),
]


@pytest.mark.parametrize("ctype,depth", CASES)
@pytest.mark.parametrize("level", [0, 1, 9])
def test_png_decoder_matches_encoder(png_check, tmp_path, ctype, depth, level):
    rng = np.random.default_rng(ctype * 100 + depth * 10 + level)
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    w, h = int(rng.integers(1, 40)), int(rng.integers(1, 30))
    palette = None
    if ctype == 3:
        palette = rng.integers(0, 256, ((1 << depth), 3))
        samples = rng.integers(0, 1 << depth, (h, w, 1))
    else:
        # mix of noise and a smooth ramp so both literal and match codes are exercised
        top = (1 << depth) - 1
        ramp = (np.arange(w)[None, :, None] * top // max(1, w - 1)) * np.ones((h, 1, chans), np.int64)
        noise = rng.integers(0, top + 1, (h, w, chans))
        samples = np.where(rng.random((h, w, chans)) < 0.5, ramp, noise)
    path = tmp_path / "in.png"
    path.write_bytes(encode_png(samples, ctype, depth, rng, level, palette, split_idat=(level == 9)))
    got, gray = _read(png_check, path, tmp_path)
    np.testing.assert_array_equal(got, expected_rgb(samples, ctype, depth, palette))
    assert gray == (ctype in (0, 4))


def test_png_writer_round_trips(png_check, tmp_path):
    from sad_gb300 import imageio
    rng = np.random.default_rng(7)
    for w, h in [(1, 1), (37, 19), (300, 250)]:  # 300x250x3 spans two stored blocks
        img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
        raw, out = tmp_path / "img.raw", tmp_path / "img.png"
        raw.write_bytes(img.tobytes())
        r = subprocess.run([png_check, "write", str(raw), str(w), str(h), str(out)], capture_output=True)
        assert r.returncode == 0
        np.testing.assert_array_equal(imageio.read_png(str(out)), img)  # independent decoder
        got, gray = _read(png_check, out, tmp_path)
        np.testing.assert_array_equal(got, img)
        assert not gray
        src = tmp_path / "py.png"
        imageio.write_png(str(src), img)
        got, _ = _read(png_check, src, tmp_path)
        np.testing.assert_array_equal(got, img)


def test_png_decoder_rejects_bad_files(png_check, tmp_path):
    rng = np.random.default_rng(3)
    good = encode_png(rng.integers(0, 256, (8, 8, 3)), 2, 8, rng)
    bad = {
        "not_png": b"GIF89a" + good[6:],
        "truncated": good[: len(good) // 2],
        "interlaced": good.replace(struct.pack(">IIBBBBB", 8, 8, 8, 2, 0, 0, 0),
                                   struct.pack(">IIBBBBB", 8, 8, 8, 2, 0, 0, 1)),
        "huge": good.replace(struct.pack(">IIBBBBB", 8, 8, 8, 2, 0, 0, 0),
                             struct.pack(">IIBBBBB", 1 << 20, 1 << 20, 8, 2, 0, 0, 0)),
    }
    for name, data in bad.items():
        p = tmp_path / f"{name}.png"
        p.write_bytes(data)
        r = subprocess.run([png_check, "read", str(p), str(tmp_path / "x.raw")], capture_output=True, text=True)
        assert r.returncode == 1, name
        assert r.stderr.strip(), name


# ---------------------------------------------------------------------------
# JPEG reading
# ---------------------------------------------------------------------------
def _test_image(h, w, grey, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    a = np.stack([128 + 100 * np.sin(x / 7 + k) * np.cos(y / 5 - k) for k in range(1 if grey else 3)], -1)
    a = np.clip(a + rng.normal(0, 6, a.shape), 0, 255).astype(np.uint8)
    return a[..., 0] if grey else a


JPEG_CASES = [  # (height, width, luma sampling, restart interval, 16-bit tables, grey, one DHT segment)
    (9, 13, (1, 1), 0, False, True, True),
    (11, 17, (1, 1), 0, False, False, False),
    (21, 33, (2, 2), 2, False, False, True),
    (16, 16, (2, 1), 0, True, False, True),
    (30, 9, (1, 2), 3, False, False, False),
    (1, 1, (2, 2), 0, False, False, True),
    (64, 80, (2, 2), 1, False, False, True),
    (40, 23, (1, 1), 7, True, True, False),
]


@pytest.mark.parametrize("h,w,sampling,restart,q16,grey,one_dht", JPEG_CASES)
def test_jpeg_decoder_matches_encoder(png_check, tmp_path, h, w, sampling, restart, q16, grey, one_dht):
    import jpeg_encode
    img = _test_image(h, w, grey, h * 31 + w)
    data, expected = jpeg_encode.encode(img, sampling=sampling, restart=restart, q16=q16, one_dht=one_dht)
    path = tmp_path / "img.jpg"
    path.write_bytes(data)
    got, gray = _read(png_check, path, tmp_path)
    assert gray == grey
    # float IDCT and colour conversion on both sides: at most a rounding step apart
    d = np.abs(got.astype(np.int64) - expected.astype(np.int64))
    assert d.max() <= 1 and d.mean() < 1e-3


def test_jpeg_decoder_segment_variants(png_check, tmp_path):
    """Fill bytes before markers, a DRI segment of 0 (no restarts), no APP0 header, unknown
    APPn segments: the same pixels as the plain file."""
    import jpeg_encode
    img = _test_image(20, 28, False, 5)
    plain, expected = jpeg_encode.encode(img, sampling=(2, 2))
    bare, _ = jpeg_encode.encode(img, sampling=(2, 2), app0=False)
    sof = plain.index(b"\xff\xc0")
    variants = {
        "fill": plain[:sof] + b"\xff\xff\xff" + plain[sof:],
        "dri0": plain[:sof] + b"\xff\xdd\x00\x04\x00\x00" + plain[sof:],
        "app1": plain[:2] + b"\xff\xe1\x00\x08Exif\x00\x00" + plain[2:],
        "no_app0": bare,
    }
    for name, data in variants.items():
        p = tmp_path / f"{name}.jpg"
        p.write_bytes(data)
        got, _ = _read(png_check, p, tmp_path)
        assert np.abs(got.astype(np.int64) - expected).max() <= 1, name


def test_jpeg_decoder_near_lossless_against_source(png_check, tmp_path):
    """Unit quantisation tables: the decode comes back to the source image (the colour
    conversion and block order checked against the pixels, not against the writer's model)."""
    import jpeg_encode
    ones = np.ones(64, np.int64)
    for sampling in [(1, 1), (2, 2)]:
        img = _test_image(48, 40, False, 1)
        data, _ = jpeg_encode.encode(img, sampling=sampling, luma_q=ones, chroma_q=ones)
        path = tmp_path / "img.jpg"
        path.write_bytes(data)
        got, _ = _read(png_check, path, tmp_path)
        mse = np.mean((got.astype(np.float64) - img) ** 2)
        assert 10 * np.log10(255.0 ** 2 / mse) > (45.0 if sampling == (1, 1) else 28.0)


def test_jpeg_decoder_rejects_bad_files(png_check, tmp_path):
    import jpeg_encode
    good, _ = jpeg_encode.encode(_test_image(16, 16, False, 2))
    sof = good.index(b"\xff\xc0")
    bad = {
        "progressive": good[:sof + 1] + b"\xc2" + good[sof + 2:],
        "truncated": good[: len(good) * 2 // 3],
        "truncated_scan": good[:-12],
        "precision12": good[:sof + 4] + b"\x0c" + good[sof + 5:],
        "no_scan": good[: good.index(b"\xff\xda")] + b"\xff\xd9",
        "too_large": good[:sof + 5] + struct.pack(">HH", 60000, 60000) + good[sof + 9:],
        # within the size limit, but far more blocks than a few hundred bytes of scan can code
        "huge": good[:sof + 5] + struct.pack(">HH", 40000, 40000) + good[sof + 9:],
    }
    for name, data in bad.items():
        p = tmp_path / f"{name}.jpg"
        p.write_bytes(data)
        r = subprocess.run([png_check, "read", str(p), str(tmp_path / "x.raw")], capture_output=True, text=True)
        assert r.returncode == 1, name
        assert r.stderr.strip(), name
    for name, needle in [("progressive", "progressive"), ("huge", "truncated"), ("truncated_scan", "truncated")]:
        r = subprocess.run([png_check, "read", str(tmp_path / f"{name}.jpg"), str(tmp_path / "x.raw")],
                           capture_output=True, text=True)
        assert needle in r.stderr, (name, r.stderr)


def test_image_readers_survive_corrupted_files(tmp_path):
    """Truncated and byte-corrupted PNG and JPEG files end in an error message or an image,
    never in a crash, with the readers built under AddressSanitizer and UBSan."""
    import jpeg_encode
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "png_check_asan")
    r = subprocess.run([cxx, "-O1", "-g", "-std=c++17", "-ffp-contract=off", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=undefined", "-I" + CLI_SRC,
                        os.path.join(ROOT, "tests", "cli", "png_check.cpp"), os.path.join(CLI_SRC, "png.cpp"),
                        os.path.join(CLI_SRC, "jpeg.cpp"), "-o", exe], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtime not available: " + r.stderr[-200:])
    rng = np.random.default_rng(0)
    jpg, _ = jpeg_encode.encode(_test_image(24, 40, False, 3), sampling=(2, 2), restart=2)
    png = encode_png(rng.integers(0, 256, (20, 30, 3)), 2, 8, rng)
    f, out = tmp_path / "f.bin", tmp_path / "f.raw"
    outcomes = {0: 0, 1: 0}
    for trial in range(300):
        b = bytearray(jpg if trial % 2 == 0 else png)
        if trial % 3 == 0:
            b = b[: rng.integers(2, len(b))]
        else:
            for _ in range(rng.integers(1, 6)):
                b[rng.integers(2, len(b))] = rng.integers(0, 256)
        f.write_bytes(bytes(b))
        r = subprocess.run([exe, "read", str(f), str(out)], capture_output=True, text=True)
        assert r.returncode in (0, 1), (trial, r.returncode, r.stderr[-800:])
        outcomes[r.returncode] += 1
    assert outcomes[1] > 0


# ---------------------------------------------------------------------------
# arguments and configuration
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def sad_cuda(sadlib):
    from sad_gb300 import build
    return build.build_cli()


def _run(exe, args, cwd, config=None):
    env = {k: v for k, v in os.environ.items() if k != "CONFIG_PATH"}
    if config is not None:
        env["CONFIG_PATH"] = str(config)
    return subprocess.run([exe, *args], cwd=cwd, env=env, capture_output=True, text=True, timeout=60)


def test_cli_help_and_defaults(sad_cuda, tmp_path):
    r = _run(sad_cuda, ["--help"], tmp_path, PACKAGED_CONFIG)
    assert r.returncode == 0
    assert r.stdout.startswith("Usage:")
    assert "--sites N             Number of sites (default: 128000)" in r.stdout
    cfg = json.load(open(PACKAGED_CONFIG))
    cfg["DEFAULT_SITES"] = 777
    cfg["PRUNE_FREQ"] = 13
    (tmp_path / "training_config.json").write_text(json.dumps(cfg))
    r = _run(sad_cuda, ["-h"], tmp_path)  # ./training_config.json when CONFIG_PATH is unset
    assert r.returncode == 0
    assert "(default: 777)" in r.stdout and "Prune frequency (default: 13)" in r.stdout


def test_cli_configuration_errors(sad_cuda, tmp_path):
    r = _run(sad_cuda, ["--help"], tmp_path)
    assert r.returncode == 1
    assert "Missing training_config.json (required)." in r.stderr
    cfg = json.load(open(PACKAGED_CONFIG))
    del cfg["INIT_RADIUS"]
    p = tmp_path / "partial.json"
    p.write_text(json.dumps(cfg))
    r = _run(sad_cuda, ["x.png"], tmp_path, p)
    assert r.returncode == 1
    assert "INIT_LOG_TAU and INIT_RADIUS must be set" in r.stderr
    cfg = json.load(open(PACKAGED_CONFIG))
    cfg["PRUNE_FREQ"] = "forty"
    p.write_text(json.dumps(cfg))
    r = _run(sad_cuda, ["--help"], tmp_path, p)
    assert r.returncode == 1 and "PRUNE_FREQ" in r.stderr


@pytest.mark.parametrize("args,needle", [
    (["--bogus"], "Unknown option: --bogus"),
    ([], "Usage:"),
    (["img.png", "--sites"], "Missing value for --sites"),
    (["img.png", "--iters", "many"], "Invalid integer for --iters"),
    (["a.png", "b.png"], "Unexpected argument: b.png"),
    (["a.png", "--render-packed"], "--render-packed is only valid in render mode"),
])
def test_cli_argument_errors(sad_cuda, tmp_path, args, needle):
    r = _run(sad_cuda, args, tmp_path, PACKAGED_CONFIG)
    assert r.returncode == 1
    assert needle in r.stdout + r.stderr


def test_cli_missing_image_fails_before_gpu_work(sad_cuda, tmp_path):
    r = _run(sad_cuda, [str(tmp_path / "missing.png")], tmp_path, PACKAGED_CONFIG)
    assert r.returncode == 1
    assert "Failed to load image" in r.stderr


def test_run_sh_backend_selection(sad_cuda, tmp_path):
    run_sh = os.path.join(ROOT, "run.sh")
    r = subprocess.run([run_sh, "--backend", "wgpu", "x.png"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "not part of this build" in r.stdout
    r = subprocess.run([run_sh, "--backend=cuda", "--help"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("Usage:")
    missing = str(tmp_path / "missing_sites.txt")
    r = subprocess.run([os.path.join(ROOT, "render.sh"), missing], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1 and "Failed to open sites TXT: " + missing in r.stderr


def test_packaged_config_matches_library_defaults(sadlib):
    """The packaged training_config.json and sad_train_config_default agree key by key."""
    import ctypes as C
    from sad_gb300 import _lib
    c = _lib.TrainConfig()
    sadlib.sad_train_config_default(C.byref(c))
    cfg = json.load(open(PACKAGED_CONFIG))
    keys = {"DEFAULT_SITES": "n_sites", "DEFAULT_MAX_SITES": "max_sites", "DEFAULT_ITERS": "iterations",
            "DEFAULT_TARGET_BPP": "target_bpp", "PRUNE_PERCENTILE": "prune_percentile",
            "PRUNE_DURING_DENSIFY": "prune_during_densify", "PRUNE_START": "prune_start",
            "PRUNE_FREQ": "prune_freq", "PRUNE_END": "prune_end", "DENSIFY_START": "densify_start",
            "DENSIFY_FREQ": "densify_freq", "DENSIFY_END": "densify_end",
            "DENSIFY_PERCENTILE": "densify_percentile", "DENSIFY_SCORE_ALPHA": "densify_score_alpha",
            "CAND_UPDATE_FREQ": "cand_update_freq", "CAND_UPDATE_PASSES": "cand_update_passes",
            "CAND_RADIUS_SCALE": "cand_radius_scale", "CAND_RADIUS_PROBES": "cand_radius_probes",
            "CAND_DOWNSCALE": "cand_downscale", "CAND_INJECT_COUNT": "cand_inject_count",
            "CAND_HILBERT_WINDOW": "cand_hilbert_window", "CAND_HILBERT_PROBES": "cand_hilbert_probes",
            "LR_POS_BASE": "lr_pos", "LR_TAU_BASE": "lr_tau", "LR_RADIUS_BASE": "lr_radius",
            "LR_COLOR_BASE": "lr_color", "LR_DIR_BASE": "lr_dir", "LR_ANISO_BASE": "lr_aniso",
            "INIT_LOG_TAU": "init_log_tau", "INIT_RADIUS": "init_radius", "BETA1": "beta1",
            "BETA2": "beta2", "EPS": "eps"}
    for k, f in keys.items():
        assert np.float32(cfg[k]) == np.float32(getattr(c, f)), k


def test_run_sh_batch_log_on_failure(sad_cuda, tmp_path):
    """A directory input runs the batch loop; an unreadable image stops it with exit 1 and a
    FAILED entry in <out-dir>/batch_<timestamp>.log (run.sh batch-mode log layout)."""
    imgs = tmp_path / "imgs"
    imgs.mkdir()
    (imgs / "broken.png").write_bytes(b"not a png")
    out = tmp_path / "out"
    r = subprocess.run([os.path.join(ROOT, "run.sh"), str(imgs), "--iters", "5", "--out-dir", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 1
    assert "Found 1 image(s)" in r.stdout and "Error processing" in r.stdout
    logs = list(out.glob("batch_*.log"))
    assert len(logs) == 1
    text = logs[0].read_text()
    assert "Total images: 1" in text and "Image: broken.png" in text
    assert "Status: FAILED (exit code: 1)" in text and "BATCH PROCESSING FAILED at image: broken.png" in text
    empty = tmp_path / "empty"
    empty.mkdir()
    r = subprocess.run([os.path.join(ROOT, "run.sh"), str(empty)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1 and "No image files found in directory" in r.stdout
