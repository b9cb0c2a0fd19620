"""Time the reference's own CUDA CLI on the benchmark workload and this library's trainer on
the identical 8-bit image (equal-PSNR speed comparison).  Prints one JSON line.

    oracle/ref/stage.sh /path/to/reference && oracle/ref/build.sh
    python oracle/ref/time_reference.py [--repeats 2] [--size 1024] [--seeds 4]
    python oracle/ref/time_reference.py --batch 64 [--iters 2000] [--workers 8]
    python oracle/ref/time_reference.py --cli-compare --size 256 --sites 4096 --iters 200

The reference binary (oracle/_ref/sad_cuda, built from the staged copy of its sources)
reads training_config.json from its working directory (baseline/_ref/sad holds the staged
one) and prints "Iter N | PSNR: x dB | Active: a/n | r it/s | t s" lines; its it/s is
iterations / seconds since the end of its initialisation.  Ours is timed the same way
(init excluded), with CUDA events around the training loop.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT]


REF_EXE = os.path.join(ROOT, "oracle", "_ref", "sad_cuda")


def run_reference(png: str, repeats: int, log_freq: int):
    exe = REF_EXE
    cwd = os.path.join(ROOT, "baseline", "_ref", "sad")
    best = None
    runs = []  # (final PSNR line, last logged PSNR with two decimals) of every repeat
    for _ in range(repeats):
        out_dir = tempfile.mkdtemp()
        t0 = time.perf_counter()
        r = subprocess.run([exe, png, "--log-freq", str(log_freq), "--out-dir", out_dir], cwd=cwd,
                           capture_output=True, text=True, timeout=1800)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(f"reference CLI failed: {r.stdout[-2000:]} {r.stderr[-2000:]}")
        its = [float(m) for m in re.findall(r"\|\s*([0-9.]+) it/s", r.stdout)]
        psnr = re.findall(r"Final PSNR: ([0-9.]+)", r.stdout)
        ttime = re.findall(r"Training time: ([0-9.]+) s", r.stdout)
        act = re.findall(r"Active: (\d+)/(\d+)", r.stdout)
        logged = re.findall(r"Iter\s+(\d+) \| PSNR: ([0-9.]+) dB", r.stdout)
        runs.append((float(psnr[-1]) if psnr else None,
                     (int(logged[-1][0]), float(logged[-1][1])) if logged else None))
        res = {"it_per_s": its[-1] if its else None, "psnr_db": float(psnr[-1]) if psnr else None,
               "training_time_s": float(ttime[-1]) if ttime else None, "wall_s": round(wall, 3),
               "active_final": int(act[-1][0]) if act else None, "log": r.stdout.splitlines()[-12:]}
        if best is None or (res["it_per_s"] or 0) > (best["it_per_s"] or 0):
            best = res
    best["psnr_runs"] = [r[0] for r in runs]
    best["last_log_psnr_runs"] = [r[1] for r in runs]  # [iteration, PSNR] of the last log line
    return best


def run_ours(img, repeats: int):
    import torch
    from sad_gb300.trainer import Trainer
    h, w = img.shape[:2]
    tr = Trainer(w, h, log_freq=0)
    tr.set_target(torch.from_numpy(img).cuda())
    from sad_gb300 import _lib
    stream = torch.cuda.ExternalStream(_lib.load().sad_trainer_stream(tr._h))
    best = None
    for _ in range(repeats + 1):  # first fit warms up
        tr.init()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        tr.run()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        res = {"it_per_s": tr.cfg.iterations / (ms / 1e3), "psnr_db": tr.psnr(),
               "training_time_s": ms / 1e3, "active_final": int(tr.sites().shape[0])}
        if best is None or res["it_per_s"] > best["it_per_s"]:
            best = res
    tr.close()
    return best


def run_batch(count: int, iters: int, workers: int):
    """The batch workload (bench.py --workload batch): the reference CLI once per image,
    sequentially (its run.sh batch mode), against this library's executor on the same
    8-bit images and iteration count."""
    import bench
    from sad_gb300 import imageio
    from sad_gb300.config import train_config
    from sad_gb300.executor import Executor
    exe = REF_EXE
    cwd = os.path.join(ROOT, "baseline", "_ref", "sad")
    imgs = bench.batch_images(count)
    d = tempfile.mkdtemp()
    pngs = []
    for k, img in enumerate(imgs):
        pngs.append(os.path.join(d, f"batch_{k:02d}.png"))
        imageio.save_image(pngs[-1], img)
    ref_psnr = []
    t0 = time.perf_counter()
    for png in pngs:
        r = subprocess.run([exe, png, "--iters", str(iters), "--log-freq", str(10 * iters), "--out-dir",
                            os.path.join(d, "out")], cwd=cwd, capture_output=True, text=True, timeout=1800)
        if r.returncode != 0:
            raise RuntimeError(f"reference CLI failed on {png}: {r.stdout[-1000:]} {r.stderr[-1000:]}")
        ref_psnr.append(float(re.findall(r"Final PSNR: ([0-9.]+)", r.stdout)[-1]))
    ref_wall = time.perf_counter() - t0
    cfg = train_config(log_freq=0, iterations=iters)
    ours = {}
    for w in (workers, 1):
        with Executor(workers=w) as ex:
            ex.submit_fit(imgs[0], config=train_config(log_freq=0, iterations=20)).result()
            order = sorted(range(len(imgs)), key=lambda i: -imgs[i].shape[0] * imgs[i].shape[1])
            t0 = time.perf_counter()
            sub = {i: ex.submit_fit(imgs[i], config=cfg) for i in order}  # largest first
            ex.wait_all()
            ours[w] = (time.perf_counter() - t0, [sub[i].result()[1] for i in range(len(imgs))])
    mean = lambda xs: round(float(np.mean(xs)), 3)  # noqa: E731
    return {"workload": f"batch of {count} images (bench.py --workload batch sizes), {iters} iterations, 1.0 bpp",
            "images": [f"{i.shape[1]}x{i.shape[0]}" for i in imgs],
            "reference_cli_sequential_wall_s": round(ref_wall, 3), "reference_psnr_mean": mean(ref_psnr),
            "ours_executor_wall_s": round(ours[workers][0], 3), "ours_executor_workers": workers,
            "ours_sequential_wall_s": round(ours[1][0], 3), "ours_psnr_mean": mean(ours[workers][1]),
            "speedup_vs_reference": round(ref_wall / ours[workers][0], 2)}


def run_cli_compare(size: int, sites: int, iters: int, repeats: int, seeds: int = 1):
    """Both command-line binaries with the same arguments on the same 8-bit image: a fit with
    a fixed site count (densify, prune and the bpp rule off), then render-only from the
    reference fit's sites file.  Best of `repeats` per binary."""
    from sad_gb300 import imageio
    from sad_gb300.synthetic import quantize_u8, synthetic_image
    d = tempfile.mkdtemp()
    pngs = []
    for sd in range(seeds):
        pngs.append(os.path.join(d, f"synthetic_{size}_s{sd}.png"))
        imageio.save_image(pngs[-1], quantize_u8(synthetic_image(size, size, seed=sd)))
    png = pngs[0]
    staged = os.path.join(ROOT, "baseline", "_ref", "sad")
    bins = {"reference": (REF_EXE, dict(os.environ)),
            "ours": (os.path.join(ROOT, "sad_gb300", "_lib", "sad_cuda"),
                     dict(os.environ, CONFIG_PATH=os.path.join(staged, "training_config.json")))}
    fit_args = ["--sites", str(sites), "--iters", str(iters), "--target-bpp", "0", "--densify-percentile", "0",
                "--prune-percentile", "0", "--log-freq", str(10 * iters)]
    out = {"workload": f"{size}x{size} synthetic (8-bit), {sites} sites fixed (densify, prune, bpp rule off), "
                       f"{iters} iterations; then render-only from the reference fit's sites"}

    def run(exe, env, args):
        r = subprocess.run([exe, *args], cwd=staged, env=env, capture_output=True, text=True, timeout=1800)
        if r.returncode != 0:
            raise RuntimeError(f"{exe} failed: {r.stdout[-1500:]} {r.stderr[-1500:]}")
        return r.stdout

    for impl in ("reference", "ours"):
        exe, env = bins[impl]
        best = None
        for k in range(repeats):
            od = os.path.join(d, f"{impl}_{k}")
            log = run(exe, env, [png, *fit_args, "--out-dir", od])
            res = {"training_time_s": float(re.findall(r"Training time: ([0-9.]+) s", log)[-1]),
                   "psnr_db": float(re.findall(r"Final PSNR: ([0-9.]+)", log)[-1]),
                   "it_per_s_log": float(re.findall(r"\|\s*([0-9.]+) it/s", log)[-1])}
            if best is None or res["training_time_s"] < best["training_time_s"]:
                best = res
        out[impl] = best
    # PSNR over all seeds (one fit each) and the PSNR trajectory of the first image
    for impl in ("reference", "ours"):
        exe, env = bins[impl]
        finals = []
        for sd, p in enumerate(pngs):
            log = run(exe, env, [p, *fit_args[:-1], str(20), "--out-dir", os.path.join(d, f"{impl}_seed{sd}")])
            finals.append(float(re.findall(r"Final PSNR: ([0-9.]+)", log)[-1]))
            if sd == 0:
                out[impl]["psnr_trajectory"] = [(int(i), float(v)) for i, v in
                                                re.findall(r"Iter +(\d+) \| PSNR: ([0-9.]+)", log)]
        out[impl]["psnr_per_seed"] = finals
        out[impl]["psnr_mean"] = round(float(np.mean(finals)), 3)
    ref_sites = os.path.join(d, "reference_0", os.path.basename(png)[:-4] + "_sites.txt")
    for impl in ("reference", "ours"):
        exe, env = bins[impl]
        best = None
        for k in range(repeats):
            log = run(exe, env, ["--render", ref_sites, "--render-target", png, "--out",
                                 os.path.join(d, f"render_{impl}_{k}.png")])
            m = re.findall(r"Candidate build: ([0-9.]+) ms \| Render: ([0-9.]+) ms", log)[-1]
            res = {"cand_ms": float(m[0]), "render_ms": float(m[1]),
                   "render_psnr_db": float(re.findall(r"Render PSNR: ([0-9.]+)", log)[-1])}
            if best is None or res["cand_ms"] + res["render_ms"] < best["cand_ms"] + best["render_ms"]:
                best = res
        out[impl]["render_only"] = best
    # file-format interoperability: each CLI renders the other's sites file
    ours_sites = os.path.join(d, "ours_0", os.path.basename(png)[:-4] + "_sites.txt")
    cross = {}
    for impl in ("reference", "ours"):
        exe, env = bins[impl]
        log = run(exe, env, ["--render", ours_sites, "--render-target", png, "--out",
                             os.path.join(d, f"cross_{impl}.png")])
        cross[f"ours_sites_rendered_by_{impl}_psnr_db"] = float(re.findall(r"Render PSNR: ([0-9.]+)", log)[-1])
    out["cross_render"] = cross
    out["speedup_training"] = round(out["reference"]["training_time_s"] / out["ours"]["training_time_s"], 2)
    ref_r, our_r = out["reference"]["render_only"], out["ours"]["render_only"]
    out["speedup_render_only"] = round((ref_r["cand_ms"] + ref_r["render_ms"]) / (our_r["cand_ms"] + our_r["render_ms"]), 2)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cli-compare", action="store_true",
                    help="both CLIs, fixed-site fit + render-only (--size, --sites, --iters)")
    ap.add_argument("--sites", type=int, default=4096)
    ap.add_argument("--batch", type=int, default=0, help="time the batch workload on this many images")
    ap.add_argument("--iters", type=int, default=2000)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--repeats", type=int, default=2)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--log-freq", type=int, default=1000)
    ap.add_argument("--seeds", type=int, default=1, help="images: synthetic seeds 0..N-1")
    ap.add_argument("--ref-exe", default=None, help="reference CLI binary (default oracle/_ref/sad_cuda)")
    ap.add_argument("--reference-only", action="store_true", help="time only the reference CLI")
    args = ap.parse_args()
    global REF_EXE
    if args.ref_exe:
        REF_EXE = os.path.abspath(args.ref_exe)
    if args.batch:
        print(json.dumps(run_batch(args.batch, args.iters, args.workers)))
        return
    if args.cli_compare:
        print(json.dumps(run_cli_compare(args.size, args.sites, args.iters, args.repeats, args.seeds)))
        return
    from sad_gb300 import imageio
    from sad_gb300.synthetic import quantize_u8, synthetic_image
    per_seed = []
    for seed in range(args.seeds):
        img = quantize_u8(synthetic_image(args.size, args.size, seed=seed))
        png = os.path.join(tempfile.mkdtemp(), f"synthetic_{args.size}_s{seed}.png")
        imageio.save_image(png, img)
        ref = run_reference(png, args.repeats, args.log_freq)
        if args.reference_only:
            per_seed.append({"seed": seed, "reference_cuda_cli": ref})
            continue
        ours = run_ours(img, args.repeats)
        per_seed.append({"seed": seed, "reference_cuda_cli": ref, "ours": ours,
                         "speedup_it_per_s": round(ours["it_per_s"] / ref["it_per_s"], 2)
                         if ref.get("it_per_s") else None})
    mean = lambda xs: round(float(np.mean(xs)), 3)  # noqa: E731
    if args.reference_only:
        print(json.dumps({"reference_exe": REF_EXE, "per_seed": per_seed,
                          "reference_it_per_s_mean": mean([p["reference_cuda_cli"]["it_per_s"] for p in per_seed]),
                          "reference_psnr_mean": mean([p["reference_cuda_cli"]["psnr_db"] for p in per_seed])}))
        return
    out = {"workload": f"{args.size}x{args.size} synthetic (8-bit), training_config.json defaults",
           "seeds": args.seeds, "per_seed": per_seed,
           "reference_it_per_s_mean": mean([p["reference_cuda_cli"]["it_per_s"] for p in per_seed]),
           "ours_it_per_s_mean": mean([p["ours"]["it_per_s"] for p in per_seed]),
           "reference_psnr_mean": mean([p["reference_cuda_cli"]["psnr_db"] for p in per_seed]),
           "ours_psnr_mean": mean([p["ours"]["psnr_db"] for p in per_seed])}
    out["speedup_it_per_s"] = round(out["ours_it_per_s_mean"] / out["reference_it_per_s_mean"], 2)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
