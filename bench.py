"""Benchmark of the GB300 voxel path tracer (one JSON line on stdout).

Default workload (configuration 2, full shading, single scene): a 256^3 fBm
volume at 35% occupancy with a 16-entry Lambert/Torrance-Sparrow palette and
2% emissive voxels, a 1024x1024 thin-lens camera, a 1024x512 sky + sun
environment importance-sampled through its CDFs, 8 bounces with Russian
roulette after 3.  One step renders the frame from reset to its 256-sample
target (268M paths); `value` is Mpaths/s with the scene resident in HBM,
timed with CUDA events on the library's stream, L2 flushed between steps.
`e2e` repeats the step through the C ABI from pinned host buffers: upload of
the volume, palette and environment image, render, readback of the image.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference path (the
reference itself is OpenGL/GLSL and cannot run here) on all host cores on a
bounded sample of the same workload.  Under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpaths/s"
UNIT = "Mpaths/s"
L2_FLUSH_BYTES = 256 << 20


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def all_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_config(args):
    from voxeltoy_gb300 import scenes as S
    return S.config2(edge=args.edge, width=args.res, height=args.res, spp=args.spp, seed=2)


def cpu_sample_rate(cfg, seconds: float, threads: int = 0) -> dict:
    """Oracle (FP32, all cores) on a band of rows at 1 sample per pixel,
    sized to about `seconds` of work; returns Mpaths/s and the sample."""
    from oracle import binding as orc
    osc = orc.Scene(cfg.voxels, cfg.palette, cfg._emissive)
    oenv = orc.Env(cfg.env_rgb) if cfg.env_rgb is not None else orc.Env()
    # two probes (a thin band, then about a second of work) give the path rate
    rows = 16
    rate = 0.0
    for probe_seconds in (0.0, 1.0):
        if probe_seconds:
            rows = int(min(cfg.height, max(16, rate * probe_seconds / cfg.width)))
        r0 = (cfg.height - rows) // 2
        t0 = time.perf_counter()
        orc.render_average(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, 1, 32, threads,
                           rows=(r0, r0 + rows))
        rate = rows * cfg.width / max(time.perf_counter() - t0, 1e-9)
    # full frame rows, then as many samples per pixel as fit the time budget
    want = rate * seconds
    band = int(min(cfg.height, max(rows, want / cfg.width)))
    spp = int(max(1, min(cfg.spp, want / (band * cfg.width))))
    r0 = (cfg.height - band) // 2
    t0 = time.perf_counter()
    orc.render_average(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, spp, 32, threads,
                       rows=(r0, r0 + band))
    dt = time.perf_counter() - t0
    paths = band * cfg.width * spp
    return {"value": paths / dt / 1e6, "seconds": dt, "paths": paths,
            "sample": f"{band} centre rows x {cfg.width} px x {spp} spp of the {cfg.width}x{cfg.height} frame "
                      f"({paths} paths, {dt:.1f} s, FP32 oracle, {threads or os.cpu_count()} threads)"}


def emissive_for_oracle(cfg):
    from voxeltoy_gb300 import _lib as L
    from oracle import binding as orc
    if cfg.scene_flags & L.VT_SCENE_AUTO_EMISSIVE:
        cand = np.flatnonzero(np.isin(cfg.voxels.ravel(), [i + 1 for i, m in enumerate(cfg.palette)
                                                            if sum(m[1]) > 0])).astype(np.int32)
        return orc.prune_emissive(cfg.voxels, cand) if cfg.scene_flags & L.VT_SCENE_PRUNE_EMISSIVE else cand
    return None


def run_reference(args, world, rank):
    """CPU restatement of the reference path on the host cores."""
    if rank != 0:
        return 0
    cfg = workload_config(args)
    cfg._emissive = emissive_for_oracle(cfg)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample_rate(cfg, 0.5, threads)
    vals, secs, sample = [], [], ""
    for _ in range(args.steps):
        r = cpu_sample_rate(cfg, args.cpu_seconds, threads)
        vals.append(r["value"])
        secs.append(r["seconds"])
        sample = r["sample"]
    value = statistics.median(vals)
    frame_paths = cfg.width * cfg.height * cfg.spp
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * frame_paths / (value * 1e6),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict(args, cfg),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "ms_per_step extrapolates the sampled rate to the full 256-spp frame",
    }
    print(json.dumps(line), flush=True)
    return 0


def config_dict(args, cfg) -> dict:
    return {"workload": f"config2 full shading: {args.edge}^3 fBm 35% occupancy, 17-entry palette "
                        f"(8 Lambert, 8 Torrance-Sparrow, 1 emissive on 2% of voxels), {args.res}^2 thin lens, "
                        f"1024x512 sky+sun env (importance sampled), 8 bounces, RR after 3, {args.spp} spp",
            "grid": args.edge, "width": args.res, "height": args.res, "spp": args.spp, "max_bounces": 8,
            "rr_start": 3, "env": [1024, 512], "paths_per_step": cfg.width * cfg.height * cfg.spp,
            "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--edge", type=int, default=256)
    ap.add_argument("--res", type=int, default=1024)
    ap.add_argument("--spp", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--kernel", type=int, default=2, help="1 plain per-pass launches, 2 persistent")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (library defaults)")
    ap.add_argument("--slots", type=int, default=0, help="path slots per launch (skips the autotuner)")
    ap.add_argument("--trace-steps", type=int, default=0, help="DDA steps between refills (with --slots)")
    ap.add_argument("--trace-bps", type=int, default=-1, help="trace blocks per SM, 0 = occupancy (with --slots)")
    ap.add_argument("--profile", action="store_true",
                    help="only warm-up and timed renders of the resident frame (for ncu captures)")
    args = ap.parse_args()
    if args.impl == "gb300" and not args.profile:
        args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    from voxeltoy_gb300 import Context, Env, Job, Scene
    from voxeltoy_gb300 import _lib as L

    torch.cuda.set_device(local)
    cfg = workload_config(args)
    pk = peaks()
    ctx = Context(local)
    ctx.set_kernel(args.kernel)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{local}")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    scene = Scene.dense(ctx, cfg.voxels, cfg.palette, flags=cfg.scene_flags)
    env = Env(ctx, cfg.env_rgb)
    job = Job(ctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    paths = cfg.width * cfg.height * cfg.spp
    tuning = {"path_slots": "default"}
    if args.slots > 0:
        ctx.set_tuning(args.slots, args.trace_bps, args.trace_steps)
        tuning = {"path_slots": args.slots, "trace_blocks_per_sm": args.trace_bps, "trace_steps": args.trace_steps,
                  "source": "command line"}
    elif not args.no_tune and args.kernel == 2:
        from voxeltoy_gb300 import autotune
        best = autotune.tune(ctx, [job], passes=cfg.spp, repeats=1, use_cache=False)
        tuning = {k: best[k] for k in ("path_slots", "trace_blocks_per_sm", "trace_steps")}
        for r in best.get("sweep", [])[:12]:
            print("tune", json.dumps(r), file=sys.stderr)
    if args.profile:
        for k in range(args.warmup + args.steps):
            job.reset()
            t0 = time.perf_counter()
            job.render(cfg.spp)
            job.synchronize()
            if k >= args.warmup:
                print(json.dumps({"profile_step_ms": 1e3 * (time.perf_counter() - t0), "paths": paths,
                                  "launches": ctx.launch_count(), "tuning": tuning}), flush=True)
        job.close(); env.close(); scene.close(); ctx.close()
        return 0

    # event counts of one full frame: the algorithmic bytes of a launch
    cnt = job.render_counted(cfg.spp).astype(np.float64)
    job.reset()
    alg_bytes = (1 * cnt[1] + 16 * cnt[2] + 8 * cnt[3] + 4 * cnt[4] + 4 * cnt[5] + 64 * cnt[0])

    def one_step():
        job.reset()
        torch.cuda.synchronize()
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        job.render(cfg.spp)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    for _ in range(args.warmup):
        one_step()
    barrier(world)
    torch.cuda.synchronize()
    times = []
    launches0 = ctx.launch_count()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            times.append(one_step())
    launches = ctx.launch_count() - launches0
    torch.cuda.synchronize()
    barrier(world)
    ms = all_max(world, float(np.mean(times)))
    value = world * paths / (ms * 1e-3) / 1e6
    launch_ms = float(np.mean(times))
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9

    # end to end through the C ABI from pinned host memory
    vox_h = torch.from_numpy(np.ascontiguousarray(cfg.voxels)).pin_memory().numpy()
    env_h = torch.from_numpy(np.ascontiguousarray(cfg.env_rgb)).pin_memory().numpy()
    out_h = torch.empty((cfg.height, cfg.width, 4), dtype=torch.float32).pin_memory().numpy()
    h2d = vox_h.nbytes + env_h.nbytes + 32 * len(cfg.palette)
    d2h = out_h.nbytes

    def e2e_step():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc = Scene.dense(ctx, vox_h, cfg.palette, flags=cfg.scene_flags)
        ev = Env(ctx, env_h)
        jb = Job(ctx, sc, ev, cfg.camera, cfg.settings, cfg.width, cfg.height)
        jb.render(cfg.spp)
        jb.readback(out=out_h)
        dt = time.perf_counter() - t0
        jb.close(); ev.close(); sc.close()
        return dt

    e2e_step()
    e2e_times = [e2e_step() for _ in range(max(1, min(args.steps, 3)))]
    e2e_s = all_max(world, float(np.mean(e2e_times)))
    e2e_value = world * paths / e2e_s / 1e6

    cpu = None
    if rank == 0 and not args.no_cpu:
        cfg._emissive = scene.emissive()
        r = cpu_sample_rate(cfg, args.cpu_seconds)
        cpu = {"value": r["value"], "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": r["sample"]}

    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text())
        if t.get("workload") == "config2" and t.get("grid") == args.edge and t.get("res") == args.res:
            traffic = t["dram_bytes_per_launch"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators of the benchmark configurations)",
        "config": config_dict(args, cfg),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": e2e_s * 1e3},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "peak_source": pk["source"], "kernel": "k_wf_trace + k_wf_shade (one frame)",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "bytes_model": "1 B/DDA cell + 16 B/palette record + 8 B/env texel eval + 4 B/CDF probe + "
                                    "4 B/emissive read + 64 B/path framebuffer"},
        "counters_per_frame": {"paths": int(cnt[0]), "dda_cells": int(cnt[1]), "palette": int(cnt[2]),
                               "env_evals": int(cnt[3]), "cdf_probes": int(cnt[4]), "emissive_reads": int(cnt[5]),
                               "segments": int(cnt[6])},
        "time_to_spp_ms": {"p50": float(np.percentile(times, 50)), "p99": float(np.percentile(times, 99))},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "tuning": tuning,
    }
    job.close(); env.close(); scene.close(); ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
