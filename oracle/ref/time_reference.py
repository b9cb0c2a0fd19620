"""Time the reference's own CUDA CLI on the benchmark workload and this library's trainer on
the identical 8-bit image (equal-PSNR speed comparison).  Prints one JSON line.

    oracle/ref/stage.sh /path/to/reference && oracle/ref/build.sh
    python oracle/ref/time_reference.py [--repeats 2] [--size 1024] [--seeds 4]
    python oracle/ref/time_reference.py --batch 64 [--iters 2000] [--workers 8]

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


def run_reference(png: str, repeats: int, log_freq: int):
    exe = os.path.join(ROOT, "oracle", "_ref", "sad_cuda")
    cwd = os.path.join(ROOT, "baseline", "_ref", "sad")
    best = None
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
        res = {"it_per_s": its[-1] if its else None, "psnr_db": float(psnr[-1]) if psnr else None,
               "training_time_s": float(ttime[-1]) if ttime else None, "wall_s": round(wall, 3),
               "active_final": int(act[-1][0]) if act else None, "log": r.stdout.splitlines()[-12:]}
        if best is None or (res["it_per_s"] or 0) > (best["it_per_s"] or 0):
            best = res
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
    exe = os.path.join(ROOT, "oracle", "_ref", "sad_cuda")
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
            t0 = time.perf_counter()
            reqs = [ex.submit_fit(img, config=cfg) for img in imgs]
            ex.wait_all()
            ours[w] = (time.perf_counter() - t0, [r.result()[1] for r in reqs])
    mean = lambda xs: round(float(np.mean(xs)), 3)  # noqa: E731
    return {"workload": f"batch of {count} images (bench.py --workload batch sizes), {iters} iterations, 1.0 bpp",
            "images": [f"{i.shape[1]}x{i.shape[0]}" for i in imgs],
            "reference_cli_sequential_wall_s": round(ref_wall, 3), "reference_psnr_mean": mean(ref_psnr),
            "ours_executor_wall_s": round(ours[workers][0], 3), "ours_executor_workers": workers,
            "ours_sequential_wall_s": round(ours[1][0], 3), "ours_psnr_mean": mean(ours[workers][1]),
            "speedup_vs_reference": round(ref_wall / ours[workers][0], 2)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", type=int, default=0, help="time the batch workload on this many images")
    ap.add_argument("--iters", type=int, default=2000)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--repeats", type=int, default=2)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--log-freq", type=int, default=1000)
    ap.add_argument("--seeds", type=int, default=1, help="images: synthetic seeds 0..N-1")
    args = ap.parse_args()
    if args.batch:
        print(json.dumps(run_batch(args.batch, args.iters, args.workers)))
        return
    from sad_gb300 import imageio
    from sad_gb300.synthetic import quantize_u8, synthetic_image
    per_seed = []
    for seed in range(args.seeds):
        img = quantize_u8(synthetic_image(args.size, args.size, seed=seed))
        png = os.path.join(tempfile.mkdtemp(), f"synthetic_{args.size}_s{seed}.png")
        imageio.save_image(png, img)
        ref = run_reference(png, args.repeats, args.log_freq)
        ours = run_ours(img, args.repeats)
        per_seed.append({"seed": seed, "reference_cuda_cli": ref, "ours": ours,
                         "speedup_it_per_s": round(ours["it_per_s"] / ref["it_per_s"], 2)
                         if ref.get("it_per_s") else None})
    mean = lambda xs: round(float(np.mean(xs)), 3)
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
