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
import math
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


def l2_copy_gbs(device: int) -> float:
    """Bandwidth of an L2-resident copy (read + write bytes; the best over
    8, 16 and 32 MiB buffers and 5 runs of 200 copies each), the denominator
    of the L2 fraction."""
    import torch
    best_gbs = 0.0
    for mib in (8, 16, 32):
        a = torch.ones(mib << 18, dtype=torch.float32, device=f"cuda:{device}")
        b = torch.empty_like(a)
        for _ in range(20):
            b.copy_(a)
        for _ in range(5):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(200):
                b.copy_(a)
            e1.record()
            e1.synchronize()
            best_gbs = max(best_gbs, 2 * a.numel() * 4 * 200 / (e0.elapsed_time(e1) * 1e-3) / 1e9)
        del a, b
    return best_gbs


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


def workload_config(args, make=None):
    """The workload's inputs; `make` = the oracle module builds the camera and
    settings without the library (the reference arm)."""
    from voxeltoy_gb300 import scenes as S
    if args.workload == "config1":
        return S.config1(edge=args.edge, width=args.res, height=args.res, spp=args.spp, seed=1, make=make)
    return S.config2(edge=args.edge, width=args.res, height=args.res, spp=args.spp, seed=2, make=make)


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
    # a frame smaller than the budget is rendered several times over
    frames = int(max(1, want / (band * cfg.width * spp)))
    r0 = (cfg.height - band) // 2
    t0 = time.perf_counter()
    for _ in range(frames):
        orc.render_average(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, spp, 32, threads,
                           rows=(r0, r0 + band))
    dt = time.perf_counter() - t0
    paths = band * cfg.width * spp * frames
    times = f" x {frames} frames" if frames > 1 else ""
    return {"value": paths / dt / 1e6, "seconds": dt, "paths": paths,
            "sample": f"{band} centre rows x {cfg.width} px x {spp} spp of the {cfg.width}x{cfg.height} frame"
                      f"{times} ({paths} paths, {dt:.1f} s, FP32 oracle, {threads or os.cpu_count()} threads)"}


def run_reference(args, world, rank):
    """CPU restatement of the reference path on the host cores.  Inputs,
    camera and settings come from the numpy generators and the oracle
    alone: this arm never loads the CUDA library."""
    if rank != 0:
        return 0
    from oracle import binding as orc
    cfg = workload_config(args, make=orc)
    # the emissive list of an auto-emissive, pruned scene (config 2); none otherwise
    cfg._emissive = orc.emissive_list(cfg.voxels, cfg.palette, prune=True) if args.workload == "config2" else None
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
        "note": f"ms_per_step extrapolates the sampled rate to the full {args.spp}-spp frame",
    }
    print(json.dumps(line), flush=True)
    return 0


def config_dict(args, cfg) -> dict:
    if args.workload == "config1":
        return {"workload": f"config1 plain method, small: {args.edge}^3 union of 8 spheres + ground slab, one "
                            f"Lambert material (albedo 0.7), constant white sky, {args.res}^2 pinhole, 4 bounces, "
                            f"no Russian roulette, {args.spp} spp",
                "grid": args.edge, "width": args.res, "height": args.res, "spp": args.spp, "max_bounces": 4,
                "paths_per_step": cfg.width * cfg.height * cfg.spp,
                "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"}
    return {"workload": f"config2 full shading: {args.edge}^3 fBm 35% occupancy, 17-entry palette "
                        f"(8 Lambert, 8 Torrance-Sparrow, 1 emissive on 2% of voxels), {args.res}^2 thin lens, "
                        f"1024x512 sky+sun env (importance sampled), 8 bounces, RR after 3, {args.spp} spp",
            "grid": args.edge, "width": args.res, "height": args.res, "spp": args.spp, "max_bounces": 8,
            "rr_start": 3, "env": [1024, 512], "paths_per_step": cfg.width * cfg.height * cfg.spp,
            "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"}


class EventTimer:
    """CUDA-event time (ms) of the work enqueued on the library's stream."""

    def __init__(self, ctx, device: int):
        import torch
        self.torch = torch
        self.stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{device}")

    def __enter__(self):
        self.e0 = self.torch.cuda.Event(enable_timing=True)
        self.e1 = self.torch.cuda.Event(enable_timing=True)
        self.e0.record(self.stream)
        return self

    def __exit__(self, *exc):
        self.e1.record(self.stream)
        self.e1.synchronize()
        self.ms = self.e0.elapsed_time(self.e1)


def batching_jobs(ctx, n: int):
    """The batching configuration: scene i from the sphere-union generator
    (seed 100 + i, edge log-uniform 32-512, occupancy U[10%, 50%]), a
    resolution from {128, 256, 512, 1024}^2, config-1 camera and shading."""
    from voxeltoy_gb300 import Job, Scene, scenes as S
    made = []
    for i in range(n):
        vox, res, seed = S.config3_scene(i)
        cfg = S.config1(edge=8, width=res, height=res, spp=64, seed=seed)
        sc = Scene.dense(ctx, vox, cfg.palette)
        made.append((sc, Job(ctx, sc, None, cfg.camera, cfg.settings, res, res), vox))
    return made


def run_batching(args, world, rank, local):
    import torch
    from voxeltoy_gb300 import Context
    spp = 64
    ctx = Context(local)
    made = batching_jobs(ctx, args.scenes)
    jobs = [m[1] for m in made]
    paths = sum(j.width * j.height for j in jobs) * spp
    from voxeltoy_gb300 import autotune
    best = autotune.tune(ctx, jobs, passes=16, repeats=1, use_cache=False,
                         grid={"path_slots": [1 << 22, 1 << 23, 1 << 24], "trace_blocks_per_sm": [0],
                               "trace_steps": [16]})
    timer = EventTimer(ctx, local)

    def reset():
        for j in jobs:
            j.reset()
        torch.cuda.synchronize()

    def batched():
        ctx.render_batch(jobs, spp, kernel=2)

    def plain_loop():                  # the reference's structure: one launch per scene and pass
        ctx.render_batch(jobs, spp, kernel=1)

    def per_scene():                   # one wavefront render per scene
        for j in jobs:
            j.render(spp)

    out = {}
    images = {}
    for name, fn, reps in (("batched", batched, args.steps), ("per_scene_wavefront", per_scene, 1),
                           ("plain_loop", plain_loop, 1)):
        times = []
        for k in range(reps + 1):
            reset()
            with timer:
                fn()
            if k:
                times.append(timer.ms)
        out[name] = {"ms": float(np.median(times)), "mpaths_s": paths / (np.median(times) * 1e-3) / 1e6}
        images[name] = [j.readback() for j in jobs]
    same = all(np.array_equal(a.view(np.uint32), b.view(np.uint32))
               for name in ("per_scene_wavefront", "plain_loop") for a, b in zip(images["batched"], images[name]))
    # end to end: upload every scene from pinned host memory, render the
    # batch, read every image back into pinned host memory
    import torch
    vox_h = [torch.from_numpy(np.ascontiguousarray(m[2])).pin_memory().numpy() for m in made]
    for sc, j, _v in made:
        j.close(); sc.close()
    from voxeltoy_gb300 import Job, Scene, scenes as S
    cfgs = [S.config1(edge=8, width=jobs[i].width, height=jobs[i].width, spp=spp, seed=100 + i)
            for i in range(len(vox_h))]
    outs = [torch.empty((c.height, c.width, 4), dtype=torch.float32).pin_memory().numpy() for c in cfgs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_jobs = []
    for vox, cfg in zip(vox_h, cfgs):
        sc = Scene.dense(ctx, vox, cfg.palette)
        e2e_jobs.append((sc, Job(ctx, sc, None, cfg.camera, cfg.settings, cfg.width, cfg.height)))
    ctx.render_batch([j for _s, j in e2e_jobs], spp, kernel=2)
    d2h = 0
    for (_s, j), dst in zip(e2e_jobs, outs):
        d2h += j.readback(out=dst).nbytes
    e2e_s = time.perf_counter() - t0
    for sc, j in e2e_jobs:
        j.close(); sc.close()
    ctx.close()
    b = out["batched"]
    return {"metric": METRIC, "value": b["mpaths_s"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": 1, "ms_per_step": b["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded batching configuration)",
            "config": {"workload": f"batching: {len(jobs)} sphere-union scenes (seed 100+i, edges 32-512 "
                                   f"log-uniform, occupancy U[10%,50%]), resolutions from {{128,256,512,1024}}^2, "
                                   f"Lambert 0.7, white sky, 4 bounces, {spp} spp, one launch",
                       "paths_per_step": paths, "voxels": int(sum(v.size for v in vox_h))},
            "batched": b, "per_scene_wavefront": out["per_scene_wavefront"], "plain_loop": out["plain_loop"],
            "batched_vs_plain": out["plain_loop"]["ms"] / b["ms"],
            "batched_vs_per_scene": out["per_scene_wavefront"]["ms"] / b["ms"],
            "identical_images": bool(same),
            "e2e": {"value": paths / e2e_s / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(sum(v.nbytes for v in vox_h)),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3},
            "tuning": {k: best[k] for k in ("path_slots", "trace_blocks_per_sm", "trace_steps")}}


def run_serving(args, world, rank, local):
    """Poisson request stream through vt_server: each request is a
    sphere-union scene (edge 64-512), a random orbit camera, a resolution
    with edge uniform in 256-1024 and an spp target log-uniform in
    16-1024; half of the requests reuse a resident scene.  Latency = arrival
    to the target sample count, read from the server's own clock plus the
    host's submission delay."""
    from voxeltoy_gb300 import Context, Scene, Server, scenes as S
    rng = np.random.default_rng(3)
    n = max(1, int(rng.poisson(args.rate * args.duration)))
    arrivals = np.sort(rng.uniform(0.0, args.duration, n))
    pool_n = 16
    pool = []
    for i in range(pool_n):
        edge = int(rng.integers(64, 513))
        pool.append(S.sphere_union(edge, None, 300 + i, occupancy=float(rng.uniform(0.1, 0.5))))
    ctx = Context(local)
    from voxeltoy_gb300 import _lib as L
    order = L.VT_SERVE_LEAST_WORK if args.order == "least-work" else L.VT_SERVE_ARRIVAL
    srv = Server(ctx, hbm_budget_bytes=60 << 30, max_active_jobs=64, passes_per_round=4, order=order,
                 quick_paths=args.quick_paths, round_paths_cap=args.round_cap)
    resident = []
    reqs = []
    for k in range(n):
        res = int(rng.integers(256, 1025))
        spp = int(round(math.exp(rng.uniform(math.log(16), math.log(1024)))))
        reuse = bool(resident) and rng.random() < 0.5
        pick = int(rng.integers(0, len(resident))) if reuse else int(rng.integers(0, pool_n))
        cam = S.orbit_camera(distance=2000.0, theta_deg=float(rng.uniform(0, 360)), phi_deg=float(rng.uniform(10, 80)))
        reqs.append((res, spp, reuse, pick, cam))
        if not reuse:
            resident.append(None)
    settings = S.physical_settings(max_bounces=4, rr_start=-1, seed=0)
    scenes = []
    tickets = []
    large = None
    if args.alongside:
        # config 5 served alongside the stream: the voxelized icosphere at
        # 2048^2 x 1024 spp, 8 bounces, submitted when the stream starts
        v, f = S.fbm_displaced_icosphere(level=8)
        big = Scene.voxelize(ctx, np.ascontiguousarray(v, np.float32), np.ascontiguousarray(f, np.uint32),
                             (1024, 1024, 1024), mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE,
                             palette=[S.lambert(0.7)])
        scenes.append(big)
        bcfg = S.config1(edge=8, width=2048, height=2048, spp=1024)
        bcfg.settings.max_bounces = 8
    t_start = time.perf_counter()
    if args.alongside:
        large = srv.submit(big, None, bcfg.camera, bcfg.settings, 2048, 2048, 1024)
    for k, (res, spp, reuse, pick, cam) in enumerate(reqs):
        wait = arrivals[k] - (time.perf_counter() - t_start)
        if wait > 0:
            time.sleep(wait)
        if reuse:
            sc = scenes[pick]
        else:
            sc = Scene.dense(ctx, pool[pick], [S.lambert(0.7)])
            scenes.append(sc)
        t_sub = time.perf_counter() - t_start
        tickets.append((srv.submit(sc, None, cam, settings, res, res, spp), t_sub - arrivals[k], res * res * spp))
    lat = []
    for t, delay, _p in tickets:
        rc = srv.wait(t, 3600.0)
        if rc != 0:
            raise RuntimeError(f"request {t} failed: {rc}")
        lat.append(delay + srv_latency(srv, t))
    large_ms = None
    if large is not None:
        rc = srv.wait(large, 3600.0)
        if rc != 0:
            raise RuntimeError(f"the large request failed: {rc}")
        large_ms = srv_latency(srv, large) * 1e3
        tickets.append((large, 0.0, 2048 * 2048 * 1024))
    t_end = time.perf_counter() - t_start
    lat = np.array(lat)
    stats = srv.stats()
    paths = sum(p for _t, _d, p in tickets)
    srv.close()
    for sc in scenes:
        sc.close()
    ctx.close()
    return {"metric": METRIC, "value": paths / t_end / 1e6, "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 0,
            "ms_per_step": t_end * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded request stream)",
            "config": {"workload": f"serving: Poisson {args.rate:g} req/s for {args.duration:g} s ({n} requests), "
                                   f"sphere-union scenes edge 64-512 (pool of {pool_n}), reuse 0.5, resolution "
                                   f"256^2-1024^2, 16-1024 spp log-uniform, 4 bounces, 60 GB admission budget, "
                                   f"admission order {args.order}, quick paths {args.quick_paths}, "
                                   f"round cap {args.round_cap}",
                       "requests": n, "offered_mpaths_s": paths / args.duration / 1e6},
            "time_to_spp_ms": {"p50": float(np.percentile(lat, 50) * 1e3), "p99": float(np.percentile(lat, 99) * 1e3),
                               "max": float(lat.max() * 1e3)},
            "server": {"completed": int(stats.completed), "failed": int(stats.failed)},
            "alongside": None if large_ms is None else
            {"request": "voxelized icosphere (1.3M triangles, 1024^3) at 2048^2 x 1024 spp, 8 bounces, "
                        "submitted with the first request of the stream", "time_to_spp_ms": large_ms},
            "e2e": {"value": paths / t_end / 1e6, "unit": UNIT,
                    "h2d_bytes_per_step": int(sum(pool[r[3]].nbytes for r in reqs if not r[2])),
                    "d2h_bytes_per_step": 0}}


def srv_latency(srv, ticket) -> float:
    """Submit-to-finish seconds of a finished request (the server's clock)."""
    import ctypes as C
    from voxeltoy_gb300 import _lib as L
    secs = C.c_double()
    L.call("vt_server_result", srv.h, ticket, None, 0, C.byref(secs))
    return secs.value


def run_voxelize(args, world, rank, local):
    """1.3M-triangle fBm-displaced icosphere, conservative voxelization into
    1024^3, then a 2048^2 render with config-1 materials and sky, 8 bounces."""
    import torch
    from voxeltoy_gb300 import Context, Job, Scene, scenes as S
    from voxeltoy_gb300 import _lib as L
    v, f = S.fbm_displaced_icosphere(level=8)
    v = np.ascontiguousarray(v, np.float32)
    f = np.ascontiguousarray(f, np.uint32)
    res = (1024, 1024, 1024)
    ctx = Context(local)
    vox_ms = []
    for k in range(args.steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc = Scene.voxelize(ctx, v, f, res, mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE,
                            palette=[S.lambert(0.7)])
        sc.info()
        torch.cuda.synchronize()
        if k:
            vox_ms.append((time.perf_counter() - t0) * 1e3)
        if k < args.steps:
            sc.close()
    check = None
    if args.check:
        from oracle import binding as orc
        want = orc.voxelize(v, f, res, L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE)
        got = sc.voxels()
        check = {"bit_exact": bool(np.array_equal(want > 0, got > 0)), "occupied": int(np.count_nonzero(got))}
    spp = args.spp if args.spp != 256 else 1024
    cfg = S.config1(edge=8, width=2048, height=2048, spp=spp)
    cfg.settings.max_bounces = 8
    job = Job(ctx, sc, None, cfg.camera, cfg.settings, 2048, 2048)
    timer = EventTimer(ctx, local)
    job.render(4)
    job.reset()
    torch.cuda.synchronize()
    with timer:
        job.render(spp)
    paths = 2048 * 2048 * spp
    img = job.readback()
    job.close(); sc.close(); ctx.close()
    return {"metric": METRIC, "value": paths / (timer.ms * 1e-3) / 1e6, "unit": UNIT, "n_gpus": world, "steps": 1,
            "warmup": 1, "ms_per_step": timer.ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded icosphere mesh)",
            "config": {"workload": f"voxelize: fBm-displaced icosphere level 8 ({len(f)} triangles) -> 1024^3 "
                                   f"conservative, then 2048^2 pinhole, Lambert 0.7, white sky, 8 bounces, {spp} spp",
                       "triangles": int(len(f))},
            "voxelize_ms": {"median": float(np.median(vox_ms)), "min": float(min(vox_ms))},
            "voxelize_mtris_s": len(f) / (np.median(vox_ms) * 1e-3) / 1e6,
            "occupancy_check": check, "image_finite": bool(np.isfinite(img).all()),
            "e2e": {"value": paths / (timer.ms * 1e-3) / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(v.nbytes + f.nbytes),
                    "d2h_bytes_per_step": int(img.nbytes)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (5; 1000 for config1 on the GPU)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--edge", type=int, default=None, help="grid edge (256; 64 for config1)")
    ap.add_argument("--res", type=int, default=None, help="image edge (1024; 256 for config1)")
    ap.add_argument("--spp", type=int, default=None, help="samples per pixel (256; 16 for config1)")
    ap.add_argument("--cpu-seconds", type=float, default=16.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--kernel", type=int, default=2, help="1 plain per-pass launches, 2 wavefront")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (library defaults)")
    ap.add_argument("--slots", type=int, default=0, help="path slots per launch (skips the autotuner)")
    ap.add_argument("--lanes", type=int, default=2, choices=[1, 2, 3, 4], help="wavefront lanes with --slots")
    ap.add_argument("--trace-steps", type=int, default=0, help="DDA steps between refills (with --slots)")
    ap.add_argument("--trace-bps", type=int, default=-1, help="trace blocks per SM, 0 = occupancy (with --slots)")
    ap.add_argument("--workload", default="config2",
                    choices=["config2", "config1", "batching", "serving", "voxelize"],
                    help="config2 (default, the headline line); config1 = the small plain case; batching = 64 uneven scenes in one launch vs "
                         "a loop of plain per-scene launches; serving = Poisson request stream through the "
                         "server; voxelize = 1.3M-triangle mesh into 1024^3, then a 2048^2 render")
    ap.add_argument("--scenes", type=int, default=64, help="batching: number of scenes")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: requests per second")
    ap.add_argument("--duration", type=float, default=5.0, help="serving: seconds of arrivals")
    ap.add_argument("--order", default="arrival", choices=["arrival", "least-work"],
                    help="serving: admission order of queued requests")
    ap.add_argument("--round-cap", type=int, default=0,
                    help="serving: at most this many paths of one request per round (0 = off)")
    ap.add_argument("--alongside", action="store_true",
                    help="serving: also serve the voxelized 1.3M-triangle icosphere at 2048^2 x 1024 spp")
    ap.add_argument("--quick-paths", type=int, default=1 << 24,
                    help="serving: requests with at most this many paths left finish in one round (0 = off)")
    ap.add_argument("--check", action="store_true", help="voxelize: compare the occupancy with the oracle")
    ap.add_argument("--profile", action="store_true",
                    help="only warm-up and timed renders of the resident frame (for ncu captures)")
    args = ap.parse_args()
    small = args.workload == "config1"
    args.edge = args.edge or (64 if small else 256)
    args.res = args.res or (256 if small else 1024)
    args.spp = args.spp or (16 if small else 256)
    args.steps = args.steps or (1000 if small and args.impl == "gb300" else 5)
    if args.impl == "gb300" and not args.profile:
        args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    from voxeltoy_gb300 import Context, Env, Job, Scene
    from voxeltoy_gb300 import _lib as L

    torch.cuda.set_device(local)
    if args.workload not in ("config2", "config1"):
        runner = {"batching": run_batching, "serving": run_serving, "voxelize": run_voxelize}[args.workload]
        line = runner(args, world, rank, local)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return 0
    cfg = workload_config(args)
    pk = peaks()
    ctx = Context(local)
    ctx.set_kernel(args.kernel)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{local}")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    scene = Scene.dense(ctx, cfg.voxels, cfg.palette, flags=cfg.scene_flags)
    env = Env(ctx, cfg.env_rgb) if cfg.env_rgb is not None else None
    job = Job(ctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    paths = cfg.width * cfg.height * cfg.spp
    tuning = {"path_slots": "default"}
    if args.slots > 0:
        ctx.set_lanes(args.lanes)
        ctx.set_tuning(args.slots, args.trace_bps, args.trace_steps)
        tuning = {"path_slots": args.slots, "trace_blocks_per_sm": args.trace_bps, "trace_steps": args.trace_steps,
                  "lanes": args.lanes, "source": "command line"}
    elif not args.no_tune and args.kernel == 2:
        from voxeltoy_gb300 import autotune
        best = autotune.tune(ctx, [job], passes=cfg.spp, repeats=1, use_cache=False)
        tuning = {k: best[k] for k in ("path_slots", "trace_blocks_per_sm", "trace_steps", "lanes")}
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
        for o in (job, env, scene, ctx):
            if o is not None:
                o.close()
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
    l2_gbs = l2_copy_gbs(local)

    # end to end through the C ABI from pinned host memory
    vox_h = torch.from_numpy(np.ascontiguousarray(cfg.voxels)).pin_memory().numpy()
    env_h = (torch.from_numpy(np.ascontiguousarray(cfg.env_rgb)).pin_memory().numpy()
             if cfg.env_rgb is not None else None)
    out_h = torch.empty((cfg.height, cfg.width, 4), dtype=torch.float32).pin_memory().numpy()
    h2d = vox_h.nbytes + (env_h.nbytes if env_h is not None else 0) + 32 * len(cfg.palette)
    d2h = out_h.nbytes

    def e2e_step():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc = Scene.dense(ctx, vox_h, cfg.palette, flags=cfg.scene_flags)
        ev = Env(ctx, env_h) if env_h is not None else None
        jb = Job(ctx, sc, ev, cfg.camera, cfg.settings, cfg.width, cfg.height)
        jb.render(cfg.spp)
        jb.readback(out=out_h)
        dt = time.perf_counter() - t0
        jb.close(); sc.close()
        if ev is not None:
            ev.close()
        return dt

    e2e_step()
    # a few whole frames; a small frame is repeated for about as long
    e2e_times = [e2e_step() for _ in range(max(1, min(args.steps, 3 if paths > 1e8 else 100)))]
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
        if (t.get("workload") == args.workload and t.get("grid") == args.edge and t.get("res") == args.res
                and t.get("spp") == args.spp):
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
                     "peak_source": pk["source"],
                     "kernel": "k_wf_shade + k_wf_hit + k_wf_regen + k_wf_trace + k_wf_accumulate (one frame = one launch)",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "bytes_model": "1 B/DDA cell + 16 B/palette record + 8 B/env texel eval + 4 B/CDF probe + "
                                    "4 B/emissive read + 64 B/path framebuffer",
                     "l2": {"achieved": achieved, "peak": l2_gbs, "unit": "GB/s", "frac": achieved / l2_gbs,
                            "peak_source": "L2-resident copy (8-32 MiB buffers) measured in this run (torch copy_)"}},
        "rates": {"gsegments_per_s": world * float(cnt[6]) / (ms * 1e-3) / 1e9,
                  "gdda_cells_per_s": world * float(cnt[1]) / (ms * 1e-3) / 1e9},
        "counters_per_frame": {"paths": int(cnt[0]), "dda_cells": int(cnt[1]), "palette": int(cnt[2]),
                               "env_evals": int(cnt[3]), "cdf_probes": int(cnt[4]), "emissive_reads": int(cnt[5]),
                               "segments": int(cnt[6]), "empty_brick_cells": int(cnt[7])},
        "time_to_spp_ms": {"p50": float(np.percentile(times, 50)), "p99": float(np.percentile(times, 99))},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "tuning": tuning,
    }
    for o in (job, env, scene, ctx):
        if o is not None:
            o.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
