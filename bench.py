"""Benchmark: SAD fit of a 1024x1024 image at 1.0 bpp with the full training_config.json
schedule (128,000 sites pruned to 8,192 over 4,000 iterations), on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --workload batch|serve      (the 64-image batch and the serving mix)

A step is one whole fit of the workload.  `value` is the training-loop throughput in
iterations/s with the image already resident in HBM (init excluded, as in the
reference's own it/s log line); `e2e` is the same metric through the host-memory entry
point sad_trainer_fit_host (image upload, init, all iterations, PSNR, download of the
active sites).  L2 is flushed (512 MB write) between steps.  Under torchrun each rank
fits its own image (replicas; no data-path collective); the barrier and the max over
ranks only bracket the timing.

--impl reference times the CPU restatement of the reference's path (the reference has
no CPU path of its own) on all host cores, on bounded samples of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WIDTH = HEIGHT = 1024
METRIC = "train iters/s @1024x1024, 1.0 bpp (training_config.json schedule)"
WORKLOAD = ("fit of a 1024x1024 RGB f32 image at 1.0 bpp: 128000 sites pruned to 8192 "
            "(bpp rule), 4000 iterations, VPT every 8, 73 prune events, K=8 candidates")
DATA = "synthetic: seeded smooth gradient + 256 Gaussian blobs + 64 convex polygons, 1024x1024"


def dist_env():
    from sad_gb300.replicas import rank_env
    e = rank_env()
    return e.world_size, e.rank, e.local_rank


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        if not getattr(self, "lines", None):
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_kernel():
    """The fused gradient kernel's committed ncu summary (DRAM bytes per launch, limiter)."""
    try:
        with open(os.path.join(ROOT, "profiles", "fused_gradients_1024.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def flush_l2(buf):
    buf.fill_(1)


def run_ours(args):
    import torch
    from sad_gb300 import replicas
    env = replicas.rank_env()
    ws, rank, local = env.world_size, env.rank, env.local_rank
    torch.cuda.set_device(local)
    replicas.init(env, "nccl")
    import sad_gb300
    from sad_gb300 import _lib
    from sad_gb300.synthetic import synthetic_image
    from sad_gb300.trainer import Trainer

    lib = _lib.load()
    img = synthetic_image(WIDTH, HEIGHT, seed=rank)
    target = torch.from_numpy(img).cuda()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    tr = Trainer(WIDTH, HEIGHT, log_freq=0, use_graphs=1)
    iters = tr.cfg.iterations
    stream = torch.cuda.ExternalStream(lib.sad_trainer_stream(tr._h))
    tr.set_target(target)

    def one_fit(timed: bool):
        tr.init()
        flush_l2(flush)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        tr.run()
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1)

    for _ in range(args.warmup):
        one_fit(False)
    replicas.barrier(env)
    torch.cuda.synchronize()
    launches0 = lib.sad_launch_count()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            times.append(one_fit(True))
    torch.cuda.synchronize()
    launches = lib.sad_launch_count() - launches0
    total_ms = replicas.max_over_ranks(env, float(sum(times)), device="cuda")
    psnr = tr.psnr()
    final_sites = tr.info().active_estimate
    value = ws * args.steps * iters / (total_ms / 1e3)

    # roofline: one instrumented fit times every fused-gradient launch with CUDA events on
    # the trainer's stream (eager launches; the kernels are the same), and samples the
    # active site count every 40 iterations
    tr.enable_timing(True)
    tr.init()
    active = []
    for end in range(40, iters + 40, 40):
        tr.run(min(end, iters))
        active.append((min(end, iters) - (end - 40), tr.info().active_estimate))
    info = tr.info()
    tr.enable_timing(False)
    grad_ms = info.gpu_ms_gradients / max(1, info.gradient_launches)
    n_buf = info.site_buffer
    mean_active = sum(k * a for k, a in active) / max(1, sum(k for k, _ in active))
    # algorithmic bytes of the fused gradient step: per pixel the target (12 B), mask (4 B)
    # and the two candidate lists (32 B); per site the gradient read-modify-write (80 B)
    alg_bytes = 48 * WIDTH * HEIGHT + 80 * n_buf
    alg_active = 48 * WIDTH * HEIGHT + 80 * mean_active
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (grad_ms / 1e3) / 1e9
    prof = profiled_kernel()
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": prof.get("dram_bytes_per_launch"),
                "limiter": prof.get("limiter"),
                # the bound the kernel does meet: L1 data-pipe wavefronts and issue, as fractions
                # of their peaks in the committed ncu capture (HBM stays at ~10%)
                "limiter_pct_of_peak": prof.get("limiter_pct_of_peak"),
                "kernel": prof.get("kernel", "fused_gradients_pre_kernel"), "launch_ms": round(grad_ms, 5),
                "algorithmic_bytes_per_launch": alg_bytes,
                "algorithmic_bytes_active_weighted": int(alg_active),
                "frac_active_weighted": round(alg_active / (grad_ms / 1e3) / 1e9 / peak, 4),
                "mean_active_sites": int(mean_active), "peak_source": peak_kind}

    # e2e: host image in pinned memory -> fit -> active sites + PSNR back
    host = torch.from_numpy(img).pin_memory().numpy()
    e2e_t = []
    sites_out = np.empty((tr.cfg.n_sites, 10), dtype=np.float32)
    for i in range(max(1, args.steps)):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sites, e2e_psnr = tr.fit_host(host, sites_out)
        e2e_t.append(time.perf_counter() - t0)
    e2e_value = ws * len(e2e_t) * iters / sum(e2e_t)
    e2e = {"value": round(e2e_value, 2), "unit": "iters/s", "h2d_bytes_per_step": int(img.nbytes),
           "d2h_bytes_per_step": int(tr.info().site_buffer * 40 + 4), "psnr_db": round(e2e_psnr, 3),
           "ms_per_fit": round(1e3 * float(np.mean(e2e_t)), 2)}
    tr.close()
    replicas.finish(env)
    if rank != 0:
        return None
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "iters/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": DATA,
        "config": {"workload": WORKLOAD, "image": f"{WIDTH}x{HEIGHT}", "target_bpp": 1.0,
                   "sites_start": 128000, "sites_final": final_sites, "iterations": iters,
                   "step": "one whole fit (training loop timed; init outside)",
                   "l2": "flushed between steps (512 MB write)", "parallelism": f"replicas x{ws}"},
        "mpix_per_s": round(value * WIDTH * HEIGHT / 1e6, 1),
        "ms_per_iteration": round(total_ms / args.steps / iters, 5),
        "psnr_db": round(psnr, 3),
        "e2e": e2e,
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline()
    return out


# The CPU sample, the same in the cpu_baseline leg and in --impl reference: iteration 0 of
# the fit runs untimed (it carries the first candidate refresh), then iterations
# 1..CPU_SAMPLE_ITERS are timed.  Until the first prune (iteration 100) all 128,000 sites are
# active, so this is the heavy start of the fit: a conservative (low) CPU rate.
CPU_SAMPLE_FIRST = 1
CPU_SAMPLE_ITERS = 300


def cpu_fit_config(threads: int):
    """The oracle's own fit config: training_config.json read by the oracle and the bpp rule
    applied by the oracle's solver (no product code on this path)."""
    import orc
    cfg_path = os.path.join(ROOT, "sad_gb300", "training_config.json")
    return orc.fit_config_json(cfg_path, WIDTH, HEIGHT, target_bpp=1.0, threads=threads)


def cpu_chunks(total: int, parts: int) -> list[int]:
    parts = max(1, parts)
    total = max(total, parts)
    return [total // parts + (1 if i < total % parts else 0) for i in range(parts)]


def cpu_sample_text(its: int, secs: float, threads: int) -> str:
    return (f"iterations {CPU_SAMPLE_FIRST}-{CPU_SAMPLE_FIRST + its - 1} of the same 1024x1024 fit "
            f"after an untimed iteration 0 ({secs:.1f} s, OpenMP x{threads})")


def cpu_baseline():
    import orc
    from sad_gb300.synthetic import synthetic_image  # numpy generator, no native code
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    img = synthetic_image(WIDTH, HEIGHT, seed=0)
    secs = sum(orc.timed_fit_sample(cpu_fit_config(threads), img, CPU_SAMPLE_FIRST, [CPU_SAMPLE_ITERS]))
    return {"value": round(CPU_SAMPLE_ITERS / secs, 4), "unit": "iters/s", "cores": threads, "kind": "port",
            "sample": cpu_sample_text(CPU_SAMPLE_ITERS, secs, threads)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    import orc
    from sad_gb300.synthetic import synthetic_image  # numpy generator, no native code
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    img = synthetic_image(WIDTH, HEIGHT, seed=0)
    cfg = cpu_fit_config(threads)
    chunks = cpu_chunks(CPU_SAMPLE_ITERS, args.steps)
    if args.warmup > 0:  # warm-up steps on a separate fit, so the timed window is the same
        orc.timed_fit_sample(cfg, img, CPU_SAMPLE_FIRST, [chunks[0]] * args.warmup)
    times = orc.timed_fit_sample(cfg, img, CPU_SAMPLE_FIRST, chunks)
    its, secs = sum(chunks), sum(times)
    value = its / secs
    return {"metric": METRIC, "value": round(value, 4), "unit": "iters/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * secs / len(times), 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": DATA, "impl": "reference",
            "config": {"workload": WORKLOAD, "image": f"{WIDTH}x{HEIGHT}",
                       "step": f"a bounded sample: iterations {CPU_SAMPLE_FIRST}-{CPU_SAMPLE_FIRST + its - 1} "
                               f"of the fit in {len(times)} timed chunks",
                       "l2": "host cores; no device involved"},
            "cpu_baseline": {"value": round(value, 4), "unit": "iters/s", "cores": threads, "kind": "port",
                             "sample": cpu_sample_text(its, secs, threads)},
            "e2e": {"value": round(value, 4), "unit": "iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference's path is CUDA-only; this is the CPU restatement of its kernels"}


# ---------------------------------------------------------------------------
# batched fits (64 images of mixed sizes) and the serving mix, through the executor
# ---------------------------------------------------------------------------
BATCH_METRIC = "batch fit wall time, 64 images (sides log-uniform 128-2048, aspect 0.5-2), 1.0 bpp, 2000 iters"
SERVE_METRIC = ("serving latency p99 ms: Poisson arrivals, 70% render-from-sites 256^2-4096^2 at 1 bpp, "
                "30% fit 256^2-1024^2 x500 iters")


def batch_specs(count: int, seed: int = 2024):
    """(width, height, seed) of the batch images: geometric-mean side log-uniform in
    [128, 2048], aspect ratio log-uniform in [0.5, 2]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        side = float(np.exp(rng.uniform(np.log(128.0), np.log(2048.0))))
        aspect = float(np.exp(rng.uniform(np.log(0.5), np.log(2.0))))
        w = int(np.clip(round(side * np.sqrt(aspect)), 64, 4096))
        h = int(np.clip(round(side / np.sqrt(aspect)), 64, 4096))
        out.append((w, h, seed + 1 + i))
    return out


def batch_images(count: int):
    from sad_gb300.synthetic import quantize_u8, synthetic_image
    return [quantize_u8(synthetic_image(w, h, seed=sd)) for w, h, sd in batch_specs(count)]


def run_batch(args):
    """The 64-image batch; the step is the whole batch: by default one lockstep batch
    (sad_batch_*), or (--batch-mode executor) all images submitted at once to the executor."""
    import torch
    from sad_gb300.config import train_config
    from sad_gb300.executor import Executor
    torch.cuda.set_device(0)
    imgs = batch_images(args.batch_images)
    cfg = train_config(log_freq=0, iterations=args.batch_iters)
    mpix_iters = sum(i.shape[0] * i.shape[1] for i in imgs) * args.batch_iters / 1e6

    # largest first (longest-processing-time order): the long fits start at once and the
    # small ones fill the gaps, which shortens the batch's makespan
    order = sorted(range(len(imgs)), key=lambda i: -imgs[i].shape[0] * imgs[i].shape[1])

    def run(workers):
        with Executor(workers=workers) as ex:
            t0 = time.perf_counter()
            sub = {i: ex.submit_fit(imgs[i], config=cfg) for i in order}
            reqs = [sub[i] for i in range(len(imgs))]
            ex.wait_all()
            wall = time.perf_counter() - t0
            res = [r.result() for r in reqs]
        return wall, [p for _, p in res], [len(s) for s, _ in res], [r.run_ms for r in reqs]

    def run_lockstep():
        """One lockstep batch: every stage one launch over all images (sad_batch_*); timed
        like the executor path, from the host images' upload to every image's sites and
        PSNR back on the host."""
        from sad_gb300.batch import Batch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with Batch([(i.shape[1], i.shape[0]) for i in imgs], config=cfg) as b:
            for i, img in enumerate(imgs):
                b.set_target(i, img)
            b.init()
            b.run()
            b.synchronize()
            psnr = [b.psnr(i) for i in range(len(imgs))]
            sites = [len(b.sites(i)) for i in range(len(imgs))]
        return time.perf_counter() - t0, psnr, sites, None  # one run for all: no per-fit times

    with Executor(workers=2) as ex:  # warm-up: kernel loading, pool growth
        for img in imgs[:2]:
            ex.submit_fit(img, config=train_config(log_freq=0, iterations=50))
        ex.wait_all()
    lockstep = args.batch_mode == "lockstep"
    if lockstep:  # warm-up of the batched kernels on a short batch of the same images
        from sad_gb300.batch import fit_batch
        fit_batch(imgs[:4], log_freq=0, iterations=50)
    with ClockSampler(0) as clk:
        walls = []
        for _ in range(args.steps):
            wall, psnr, sites, run_ms = run_lockstep() if lockstep else run(args.workers)
            walls.append(wall)
    seq_wall = run(1)[0] if args.batch_sequential else None
    exec_wall = run(args.workers)[0] if (lockstep and args.batch_compare) else None
    wall = float(np.median(walls))
    return {
        "metric": BATCH_METRIC, "value": round(wall, 3), "unit": "s", "n_gpus": 1, "steps": args.steps,
        "warmup": 1, "ms_per_step": round(1e3 * wall, 1), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded gradient + blobs + polygons per image, quantised to 8 bits",
        "config": {"workload": f"{len(imgs)} fits, sizes {min(i.shape[1] for i in imgs)}-"
                               f"{max(i.shape[1] for i in imgs)} wide, 1.0 bpp, {args.batch_iters} iterations "
                               f"each, " + ("lockstep batch (one launch per stage over all images, graph "
                                           "replays)" if lockstep else f"{args.workers} executor workers"),
                   "images": [f"{i.shape[1]}x{i.shape[0]}" for i in imgs]},
        "mpix_iters_per_s": round(mpix_iters / wall, 1),
        "images_per_s": round(len(imgs) / wall, 3),
        "sequential_wall_s": None if seq_wall is None else round(seq_wall, 3),
        "executor_wall_s": None if exec_wall is None else round(exec_wall, 3),
        "psnr_db_mean": round(float(np.mean(psnr)), 3), "sites_final_total": int(sum(sites)),
        "fit_run_ms": None if run_ms is None else {"p50": round(float(np.median(run_ms)), 1),
                                                   "max": round(float(np.max(run_ms)), 1)},
        "e2e": {"value": round(wall, 3), "unit": "s", "h2d_bytes_per_step": int(sum(i.nbytes for i in imgs)),
                "d2h_bytes_per_step": int(40 * sum(sites) + 4 * len(imgs))},
        "clocks": clk.summary(),
    }


def serve_requests(count: int, seed: int):
    """Seeded request mix: 70% renders (square side log-uniform 256..4096, sites at 1 bpp),
    30% fits (side log-uniform 256..1024, snapped to a pool of six sizes, 500 iterations)."""
    rng = np.random.default_rng(seed)
    reqs = []
    pool = [256, 320, 448, 576, 768, 1024]
    for i in range(count):
        if rng.random() < 0.7:
            side = int(round(np.exp(rng.uniform(np.log(256), np.log(4096)))))
            reqs.append(("render", side, i))
        else:
            side = float(np.exp(rng.uniform(np.log(256), np.log(1024))))
            reqs.append(("fit", min(pool, key=lambda p: abs(np.log(p / side))), i))
    return reqs


def render_sites(side: int, seed: int):
    rng = np.random.default_rng(seed)
    n = max(1, round(side * side / 128))
    s = np.zeros((n, 10), np.float32)
    s[:, 0:2] = np.floor(rng.uniform(0, side, (n, 2))) + 0.25
    s[:, 2], s[:, 3] = 5.0, 4.0
    s[:, 4:7] = rng.uniform(0, 1, (n, 3))
    th = rng.uniform(0, np.pi, n)
    s[:, 7], s[:, 8] = np.cos(th), np.sin(th)
    s[:, 9] = np.clip(rng.normal(0, 0.42, n), -4, 4)
    return s


def run_serve(args):
    import torch
    from sad_gb300.config import train_config
    from sad_gb300.synthetic import quantize_u8, synthetic_image
    torch.cuda.set_device(0)
    rates = [float(r) for r in args.serve_rates.split(",")]
    fit_cfg = train_config(log_freq=0, iterations=500)
    fit_imgs = {s: quantize_u8(synthetic_image(s, s, seed=s)) for s in (256, 320, 448, 576, 768, 1024)}
    budget = int(args.serve_budget_gb * (1 << 30))
    rows = serve_sweep(args, rates, args.workers, budget, fit_cfg, fit_imgs, args.serve_max_fits)
    seq_rows = serve_sweep(args, rates, 1, budget, fit_cfg, fit_imgs, 0) if args.serve_sequential else None
    top = rows[-1]
    return {
        "metric": SERVE_METRIC, "value": top["p99_ms"], "unit": "ms", "n_gpus": 1, "steps": len(rates),
        "warmup": 1, "ms_per_step": None, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: random 1-bpp site sets for renders, seeded synthetic images for fits",
        "config": {"workload": f"{args.serve_count} requests per rate, Poisson arrivals at {rates} /s, "
                               f"{args.workers} workers, at most {args.serve_max_fits or 'any'} fits at once, "
                               f"HBM budget {args.serve_budget_gb} GB",
                   "latency": "submission to results in host memory"},
        "rates": rows,
        "sequential_rates": seq_rows,
        "e2e": {"value": top["p99_ms"], "unit": "ms", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
    }


def serve_sweep(args, rates, workers, budget, fit_cfg, fit_imgs, max_fits):
    """The request streams of every rate through one executor of `workers` workers."""
    from sad_gb300.config import train_config
    from sad_gb300.executor import Executor
    sites_cache = {}
    rows = []
    with Executor(workers=workers, hbm_budget_bytes=budget, max_running_fits=max_fits) as ex:
        for kind, side, i in serve_requests(8, 99):  # warm-up
            if kind == "fit":
                ex.submit_fit(fit_imgs[side], config=train_config(log_freq=0, iterations=50))
            else:
                ex.submit_render(render_sites(min(side, 1024), i), min(side, 1024), min(side, 1024))
        ex.wait_all()
        for ri, rate in enumerate(rates):
            reqs = serve_requests(args.serve_count, 1000 + ri)
            gaps = np.random.default_rng(7 + ri).exponential(1.0 / rate, len(reqs))
            subs, kinds = [], []
            t0 = time.perf_counter()
            due = t0
            for (kind, side, i), gap in zip(reqs, gaps):
                due += gap
                delay = due - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                if kind == "fit":
                    subs.append(ex.submit_fit(fit_imgs[side], config=fit_cfg))
                else:
                    if (side, i) not in sites_cache:
                        sites_cache[(side, i)] = render_sites(side, i)
                    subs.append(ex.submit_render(sites_cache[(side, i)], side, side))
                kinds.append(kind)
            ex.wait_all()
            elapsed = time.perf_counter() - t0
            lat = {"fit": [], "render": []}
            fit_psnr = []
            for k, r in zip(kinds, subs):
                assert r.res.status == 0, r.res.message
                lat[k].append(r.queue_ms + r.run_ms)
                if k == "fit":
                    fit_psnr.append(float(r.res.psnr))
            subs.clear()
            sites_cache.clear()
            allv = lat["fit"] + lat["render"]
            row = {"rate_per_s": rate, "requests": len(allv), "completed_per_s": round(len(allv) / elapsed, 2),
                   "p50_ms": round(float(np.percentile(allv, 50)), 1),
                   "p99_ms": round(float(np.percentile(allv, 99)), 1)}
            if fit_psnr:
                row["fit_psnr_mean_db"] = round(float(np.mean(fit_psnr)), 2)
            for k in ("render", "fit"):
                if lat[k]:
                    row[f"{k}_p50_ms"] = round(float(np.percentile(lat[k], 50)), 1)
                    row[f"{k}_p99_ms"] = round(float(np.percentile(lat[k], 99)), 1)
            rows.append(row)
    return rows


def run_profile_batch(args):
    """The batch workload as one lockstep batch, for ncu: graph replays up to
    --profile-iters, then --profile-window eager iterations (every kernel its own launch)
    inside the NVTX range "late" (select them with ncu --nvtx --nvtx-include "late/");
    nothing is timed.  With --profile-window 0 every iteration runs eager."""
    import torch
    from sad_gb300.batch import Batch
    from sad_gb300.config import train_config
    torch.cuda.set_device(0)
    imgs = batch_images(args.batch_images)
    window = args.profile_window
    cfg = train_config(log_freq=0, iterations=args.batch_iters, use_graphs=1 if window > 0 else 0)
    with Batch([(i.shape[1], i.shape[0]) for i in imgs], config=cfg) as b:
        for i, img in enumerate(imgs):
            b.set_target(i, img)
        b.init()
        b.run(args.profile_iters)
        b.synchronize()
        if window > 0:
            b.enable_timing(True)  # eager launches from here on
            torch.cuda.nvtx.range_push("late")
            b.run(min(args.batch_iters, args.profile_iters + window))
            b.synchronize()
            torch.cuda.nvtx.range_pop()
    print(json.dumps({"mode": "profile", "workload": "batch", "iterations": args.profile_iters,
                      "window": window}))


def run_profile(args):
    """Eager (graph-free) fit of the workload for `--profile-iters` iterations, so every
    kernel is a separate launch for ncu; nothing is timed.  --profile-sites N fits N sites
    with neither pruning nor densification instead: the site density of a later phase of
    the same fit (8192: its last quarter) in a short run."""
    import torch
    from sad_gb300.synthetic import synthetic_image
    from sad_gb300.trainer import Trainer
    img = synthetic_image(WIDTH, HEIGHT, seed=0)
    extra = {}
    if args.profile_sites > 0:
        extra = dict(n_sites=args.profile_sites, max_sites=args.profile_sites, target_bpp=0.0,
                     prune_percentile=0.0, densify=0)
    tr = Trainer(WIDTH, HEIGHT, log_freq=0, use_graphs=0, **extra)
    tr.set_target(torch.from_numpy(img).cuda())
    tr.init()
    tr.run(args.profile_iters)
    torch.cuda.synchronize()
    print(json.dumps({"mode": "profile", "iterations": args.profile_iters, "psnr_db": tr.psnr()}))
    tr.close()
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="bench", choices=["bench", "profile"])
    ap.add_argument("--profile-iters", type=int, default=200)
    ap.add_argument("--profile-sites", type=int, default=0)
    ap.add_argument("--profile-window", type=int, default=0,
                    help="profile mode, batch workload: eager iterations after --profile-iters")
    ap.add_argument("--workload", default="fit", choices=["fit", "batch", "serve"],
                    help="fit: the 1024x1024 headline fit; batch: 64 mixed-size fits through the "
                         "executor; serve: the Poisson render/fit mix")
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--batch-images", type=int, default=64)
    ap.add_argument("--batch-iters", type=int, default=2000)
    ap.add_argument("--batch-sequential", action="store_true", help="also time the batch with one worker")
    ap.add_argument("--batch-mode", default="lockstep", choices=["lockstep", "executor"])
    ap.add_argument("--batch-compare", action="store_true", help="lockstep: also time the executor path")
    ap.add_argument("--serve-rates", default="5,10,20,40")
    ap.add_argument("--serve-count", type=int, default=120)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-max-fits", type=int, default=2,
                    help="at most this many fits run at once in the serving executor (0: no cap)")
    ap.add_argument("--serve-sequential", action="store_true",
                    help="also run the same request streams with one worker (requests one at a time)")
    args = ap.parse_args()
    if args.mode == "profile":
        run_profile_batch(args) if args.workload == "batch" else run_profile(args)
        return
    if args.workload != "fit":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "workload": args.workload,
                              "unavailable": "the reference fits one image per process; its batch timing "
                                             "is oracle/ref/time_reference.py --batch"}), flush=True)
            return
        out = run_batch(args) if args.workload == "batch" else run_serve(args)
        print(json.dumps(out), flush=True)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
