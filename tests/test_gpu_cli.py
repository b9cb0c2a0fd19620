"""The sad_cuda-compatible command-line host end to end on the GPU: a fit writes the render and
the sites TXT (backends/cuda/src/sad_cuda.cu:2480-2533 output names and log lines), the TXT
renders back through --render with a PSNR against the source image, and the init modes
(per-pixel, from sites), the mask and the SSIM log run.  The fits are deterministic, so two
identical runs must write byte-identical sites files."""
import os
import re
import subprocess

import numpy as np
import pytest

from sad_gb300 import imageio, sites_io
from sad_gb300.synthetic import synthetic_image

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CONFIG = os.path.join(ROOT, "sad_gb300", "training_config.json")


@pytest.fixture(scope="module")
def sad_cuda(cuda):
    from sad_gb300 import build
    return build.build_cli()


@pytest.fixture(scope="module")
def image(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    img = synthetic_image(96, 80, seed=5)
    path = d / "synth.png"
    imageio.write_png(str(path), np.round(np.clip(img, 0, 1) * 255).astype(np.uint8))
    return path


def _run(exe, args, cwd):
    env = dict(os.environ, CONFIG_PATH=CONFIG)
    r = subprocess.run([exe, *args], cwd=cwd, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def _fit(exe, image, out_dir, *extra):
    return _run(exe, [str(image), "--iters", "60", "--sites", "600", "--log-freq", "20",
                      "--out-dir", str(out_dir), *extra], out_dir.parent)


def test_cli_fit_then_render(sad_cuda, image, tmp_path):
    out = tmp_path / "results"
    log = _fit(sad_cuda, image, out)
    assert "Training | backend=cuda | image=96x80 | sites=600/600 | iters=60" in log
    assert "Schedule | init=gradient" in log
    iters = re.findall(r"Iter +(\d+) \| PSNR: ([0-9.]+) dB \| Active: (\d+)/(\d+)", log)
    assert [int(i[0]) for i in iters] == [0, 20, 40, 59]
    final = float(re.search(r"Final PSNR: ([0-9.]+) dB \(best ([0-9.]+)\)", log).group(1))
    assert final > 22.0
    png, txt = out / "synth.png", out / "synth_sites.txt"
    assert f"Saved: {png}" in log and f"Saved: {txt}" in log
    rendered = imageio.read_png(str(png))
    assert rendered.shape == (80, 96, 3)
    sites, w, h = sites_io.load_sites(str(txt))
    assert (w, h) == (96, 80)
    assert sites.shape[0] == int(iters[-1][2])

    log = _run(sad_cuda, ["--render", str(txt), "--render-target", str(image)], tmp_path)
    assert f"Loaded {sites.shape[0]} sites" in log and "Render size: 96x80" in log
    psnr = float(re.search(r"Render PSNR: ([0-9.]+) dB", log).group(1))
    assert psnr > final - 1.0
    assert re.search(r"Candidate build: [0-9.]+ ms \| Render: [0-9.]+ ms", log)
    back = imageio.read_png(str(tmp_path / "results" / "synth_sites_render.png"))
    assert back.shape == (80, 96, 3)
    # the training render and the re-render see the same sites: most pixels agree closely
    assert np.mean(np.abs(back.astype(int) - rendered.astype(int)) <= 8) > 0.95


def test_cli_fits_are_reproducible(sad_cuda, image, tmp_path):
    a, b = tmp_path / "a", tmp_path / "b"
    _fit(sad_cuda, image, a)
    _fit(sad_cuda, image, b)
    assert (a / "synth_sites.txt").read_bytes() == (b / "synth_sites.txt").read_bytes()
    assert (a / "synth.png").read_bytes() == (b / "synth.png").read_bytes()


def test_cli_init_modes_mask_and_ssim(sad_cuda, image, tmp_path):
    small = tmp_path / "small.png"
    imageio.write_png(str(small), (synthetic_image(32, 24, seed=2) * 255).round().clip(0, 255).astype(np.uint8))
    log = _run(sad_cuda, [str(small), "--init-per-pixel", "--iters", "20", "--log-freq", "10",
                          "--out-dir", str(tmp_path / "pp")], tmp_path)
    assert "sites=768/768" in log and "init=per-pixel" in log
    assert float(re.search(r"Final PSNR: ([0-9.]+)", log).group(1)) > 25.0

    first = tmp_path / "first"
    _fit(sad_cuda, image, first)
    log = _run(sad_cuda, [str(image), "--init-from-sites", str(first / "synth_sites.txt"), "--iters", "20",
                          "--log-freq", "10", "--out-dir", str(tmp_path / "again")], tmp_path)
    assert "init=sites" in log
    n_first = sites_io.load_sites(str(first / "synth_sites.txt"))[0].shape[0]
    assert f"sites={n_first}/{n_first}" in log

    mask = np.zeros((80, 96), np.uint8)
    mask[:, :48] = 255
    mpath = tmp_path / "mask.png"
    imageio.write_png(str(mpath), mask)
    log = _fit(sad_cuda, image, tmp_path / "masked", "--mask", str(mpath), "--ssim")
    assert "mask=yes" in log
    ssim = [float(s) for s in re.findall(r"\| SSIM: ([0-9.]+)", log)]
    assert len(ssim) == 4 and 0.0 < ssim[-1] <= 1.0
    assert re.search(r"Final SSIM: [0-9.]+ \(best [0-9.]+\)", log)


def test_run_sh_batch_mode(sad_cuda, tmp_path):
    imgs = tmp_path / "imgs"
    imgs.mkdir()
    import jpeg_encode
    for i, (w, h) in enumerate([(48, 40), (40, 56)]):
        img = np.round(np.clip(synthetic_image(w, h, seed=10 + i), 0, 1) * 255).astype(np.uint8)
        if i == 0:
            imageio.write_png(str(imgs / f"im{i}.png"), img)
        else:  # run.sh batches png, jpg and jpeg files
            (imgs / f"im{i}.jpg").write_bytes(jpeg_encode.encode(img, sampling=(2, 2))[0])
    out = tmp_path / "out"
    r = subprocess.run([os.path.join(ROOT, "run.sh"), str(imgs), "--iters", "30", "--sites", "200",
                        "--log-freq", "10", "--out-dir", str(out)],
                       capture_output=True, text=True, timeout=600, env=dict(os.environ, CONFIG_PATH=CONFIG))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Processed 2 image(s) successfully." in r.stdout
    text = next(out.glob("batch_*.log")).read_text()
    assert text.count("Status: SUCCESS") == 2
    assert len(re.findall(r"PSNR: [0-9.]+ dB", text)) == 2
    assert len(re.findall(r"Active sites: \d+/\d+", text)) == 2
    for i in range(2):
        assert (out / f"im{i}.png").exists() and (out / f"im{i}_sites.txt").exists()


def test_cli_fits_jpeg_like_its_decoded_pixels(sad_cuda, tmp_path):
    """A JPEG input fits exactly like a PNG holding the pixels the host's JPEG reader decodes
    (read here through tests/cli/png_check.cpp, built from the same reader source)."""
    import shutil
    import jpeg_encode
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = os.path.join(ROOT, "sad_gb300", "cli")
    check = str(tmp_path / "png_check")
    subprocess.run([cxx, "-O1", "-std=c++17", "-ffp-contract=off", "-I" + src,
                    os.path.join(ROOT, "tests", "cli", "png_check.cpp"), os.path.join(src, "png.cpp"),
                    os.path.join(src, "jpeg.cpp"), "-o", check], check=True)
    img = np.round(np.clip(synthetic_image(64, 48, seed=9), 0, 1) * 255).astype(np.uint8)
    data, model = jpeg_encode.encode(img, sampling=(2, 1))
    jpg, png, raw = tmp_path / "photo.jpg", tmp_path / "photo_png.png", tmp_path / "photo.raw"
    jpg.write_bytes(data)
    subprocess.run([check, "read", str(jpg), str(raw)], check=True)
    head, body = raw.read_bytes().split(b"\n", 1)
    decoded = np.frombuffer(body, np.uint8).reshape(48, 64, 3)
    assert np.abs(decoded.astype(np.int64) - model).max() <= 1
    imageio.write_png(str(png), decoded)
    log = _fit(sad_cuda, jpg, tmp_path / "a")
    assert "image=64x48" in log
    _fit(sad_cuda, png, tmp_path / "b")
    a = (tmp_path / "a" / "photo_sites.txt").read_bytes()
    b = (tmp_path / "b" / "photo_png_sites.txt").read_bytes()
    assert a == b
    assert imageio.read_png(str(tmp_path / "a" / "photo.png")).shape == (48, 64, 3)


def test_cli_packed_psnr_and_render_packed(sad_cuda, image, tmp_path):
    out = tmp_path / "res"
    log = _fit(sad_cuda, image, out, "--packed-psnr")
    final = float(re.search(r"Final PSNR: ([0-9.]+)", log).group(1))
    packed = float(re.search(r"Packed inference PSNR: ([0-9.]+) dB", log).group(1))
    assert final - 1.5 < packed <= final + 0.1
    assert (out / "synth_packed.png").exists()
    txt = out / "synth_sites.txt"
    log = _run(sad_cuda, ["--render", str(txt), "--render-packed", "--render-target", str(image),
                          "--out", str(tmp_path / "packed_render.png")], tmp_path)
    n = sites_io.load_sites(str(txt))[0].shape[0]
    assert f"Packed inference sites: {n} x 16 bytes" in log
    psnr = float(re.search(r"Render PSNR: ([0-9.]+) dB", log).group(1))
    assert psnr > packed - 1.0
    assert imageio.read_png(str(tmp_path / "packed_render.png")).shape == (80, 96, 3)


def test_cli_renders_json_sites_like_txt(sad_cuda, image, tmp_path):
    """The reference's JSON sites layout (sad_cuda.cu:340-389: image_width/image_height,
    sites[] of pos, color, log_tau, radius, aniso_dir, log_aniso) renders exactly as the
    same sites in TXT form."""
    import json
    out = tmp_path / "fit"
    _fit(sad_cuda, image, out)
    txt = out / "synth_sites.txt"
    sites, w, h = sites_io.load_sites(str(txt))
    doc = {"image_width": w, "image_height": h,
           "sites": [{"pos": [float(s[0]), float(s[1])], "log_tau": float(s[2]), "radius": float(s[3]),
                      "color": [float(s[4]), float(s[5]), float(s[6])], "aniso_dir": [float(s[7]), float(s[8])],
                      "log_aniso": float(s[9])} for s in sites]}
    js = tmp_path / "sites.json"
    js.write_text(json.dumps(doc))
    _run(sad_cuda, ["--render", str(txt), "--out", str(tmp_path / "a.png")], tmp_path)
    _run(sad_cuda, ["--render", str(js), "--out", str(tmp_path / "b.png")], tmp_path)
    np.testing.assert_array_equal(imageio.read_png(str(tmp_path / "a.png")), imageio.read_png(str(tmp_path / "b.png")))
