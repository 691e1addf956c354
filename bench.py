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


def l2_read_gbs(ctx) -> dict:
    """L2 read bandwidth: the best of five single launches, each sweeping a
    32 MiB buffer (a quarter of L2) 1000 times with L1-bypassing loads
    (vt_diag_l2_read_bandwidth), the denominator of the L2 fraction."""
    best = max(ctx.l2_read_bandwidth(32 << 20, 1000) for _ in range(5))
    return {"gbs": best, "source": "one kernel launch reading a 32 MiB L2-resident buffer 1000 times "
                                   "(ld.global.cg, best of 5), measured in this run"}


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


def image_digest(img: np.ndarray) -> str:
    import hashlib
    return hashlib.blake2b(np.ascontiguousarray(img).view(np.uint8), digest_size=16).hexdigest()


def rel_rmse(got: np.ndarray, ref: np.ndarray) -> dict:
    """Relative RMSE of RGB over the pixels finite in both images:
    sqrt(mean((got - ref)^2)) / sqrt(mean(ref^2))."""
    g = got[..., :3].astype(np.float64)
    r = ref[..., :3].astype(np.float64)
    ok = np.isfinite(g).all(-1) & np.isfinite(r).all(-1)
    err = float(np.sqrt(np.mean((g[ok] - r[ok]) ** 2)) / max(np.sqrt(np.mean(r[ok] ** 2)), 1e-300))
    return {"rel_rmse": err, "pixels": int(ok.size), "nonfinite_pixels": int((~ok).sum())}


def rmse_vs_fp64(cfg, img: np.ndarray, spp: int, rows, emissive=None, noise=None) -> dict:
    """The FP64 oracle's image of rows [r0, r1) of `cfg`'s frame at `spp`
    samples per pixel (the same counter-based random streams), against the
    same rows of the GPU's image: the arithmetic error of the FP32 path.
    The oracle is the checker here; nothing it computes is timed."""
    from oracle import binding as orc
    r0, r1 = rows
    osc = orc.Scene(cfg.voxels, cfg.palette, emissive)
    oenv = orc.Env(cfg.env_rgb) if cfg.env_rgb is not None else orc.Env()
    t0 = time.perf_counter()
    ref, _ = orc.render_average(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, spp, 64, rows=(r0, r1),
                                noise=noise)
    rec = rel_rmse(img[r0:r1], ref[r0:r1])
    rec.update(frame=f"{cfg.width}x{cfg.height}", rows=[int(r0), int(r1)], spp=int(spp),
               paths=int((r1 - r0) * cfg.width * spp), oracle_s=round(time.perf_counter() - t0, 2))
    return rec


def batching_jobs(ctx, n: int):
    """The batching configuration: scene i from the sphere-union generator
    (seed 100 + i, edge log-uniform 32-512, occupancy U[10%, 50%]), a
    resolution from {128, 256, 512, 1024}^2, config-1 camera and shading."""
    from voxeltoy_gb300 import Job, Scene, scenes as S
    made = []
    for i in range(n):
        vox, res, seed = S.config3_scene(i)
        cfg = S.config1(edge=8, width=res, height=res, spp=64, seed=seed)
        cfg.voxels = vox
        sc = Scene.dense(ctx, vox, cfg.palette)
        made.append((sc, Job(ctx, sc, None, cfg.camera, cfg.settings, res, res), cfg))
    return made


def batching_record(ctx, n_scenes: int, steps: int, rmse_scenes: int = 4, e2e: bool = True) -> dict:
    """Config 3: n uneven scenes in one wavefront launch (batched) against one
    wavefront launch per scene and against the reference's structure (the
    per-pixel kernel, one launch per scene and pass), identical images in all
    three forms; the relative RMSE of the batched images of the scenes with
    the largest grids (and the smallest) against the FP64 oracle."""
    import torch
    from voxeltoy_gb300 import autotune
    spp = 64
    made = batching_jobs(ctx, n_scenes)
    jobs = [m[1] for m in made]
    paths = sum(j.width * j.height for j in jobs) * spp
    best = autotune.tune(ctx, jobs, passes=16, repeats=1, use_cache=False,
                         grid={"path_slots": [1 << 24, 1 << 25], "trace_blocks_per_sm": [0],
                               "trace_steps": [16, 32], "lanes": [2, 3], "brick_shape": [(2, 2, 2)],
                               "queue_chunk": [128, 64], "refill_min": [0], "trace_form_steps": []})
    timer = EventTimer(ctx, ctx_device(ctx))

    def reset():
        for j in jobs:
            j.reset()
        torch.cuda.synchronize()

    forms = (("batched", lambda: ctx.render_batch(jobs, spp, kernel=2), steps),
             ("per_scene_wavefront", lambda: [j.render(spp) for j in jobs], 1),
             ("plain_loop", lambda: ctx.render_batch(jobs, spp, kernel=1), 1))
    out, digests, rmse_imgs = {}, {}, {}
    by_edge = sorted(range(len(made)), key=lambda k: made[k][2].voxels.shape[0])
    picks = sorted(set(by_edge[-(rmse_scenes - 1):] + by_edge[:1])) if rmse_scenes > 0 else []
    for name, fn, reps in forms:
        times = []
        for k in range(reps + 1):
            reset()
            with timer:
                fn()
            if k:
                times.append(timer.ms)
        ms = float(np.median(times))
        out[name] = {"ms": ms, "mpaths_s": paths / (ms * 1e-3) / 1e6}
        imgs = [j.readback() for j in jobs]
        digests[name] = [image_digest(a) for a in imgs]
        if name == "batched":
            rmse_imgs = {k: imgs[k] for k in picks}
        del imgs
    same = digests["batched"] == digests["per_scene_wavefront"] == digests["plain_loop"]
    rmse = []
    for k in picks:
        cfg = made[k][2]
        band = min(32, cfg.height)
        r0 = (cfg.height - band) // 2
        rec = rmse_vs_fp64(cfg, rmse_imgs[k], spp, (r0, r0 + band))
        rec.update(scene=k, grid=int(cfg.voxels.shape[0]))
        rmse.append(rec)
    rec = {"scenes": len(jobs), "spp": spp, "paths": int(paths),
           "voxels": int(sum(m[2].voxels.size for m in made)),
           "batched": out["batched"], "per_scene_wavefront": out["per_scene_wavefront"],
           "plain_loop": out["plain_loop"],
           "batched_vs_plain": out["plain_loop"]["ms"] / out["batched"]["ms"],
           "batched_vs_per_scene": out["per_scene_wavefront"]["ms"] / out["batched"]["ms"],
           "identical_images": bool(same), "rmse_vs_fp64": rmse,
           "tuning": {k: best[k] for k in ("path_slots", "trace_blocks_per_sm", "trace_steps", "lanes", "queue_chunk")}}
    vox_h = [torch.from_numpy(np.ascontiguousarray(m[2].voxels)).pin_memory().numpy() for m in made] if e2e else []
    cfgs = [m[2] for m in made]
    for sc, j, _c in made:
        j.close(); sc.close()
    if e2e:
        # upload every scene from pinned host memory, render the batch, read
        # every image back into pinned host memory
        from voxeltoy_gb300 import Job, Scene
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
        rec["e2e"] = {"value": paths / e2e_s / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(sum(v.nbytes for v in vox_h)),
                      "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3}
    return rec


def ctx_device(ctx) -> int:
    import torch
    return torch.cuda.current_device()


def run_batching(args, world, rank, local):
    from voxeltoy_gb300 import Context
    ctx = Context(local)
    b = batching_record(ctx, args.scenes, args.steps)
    ctx.close()
    return {"metric": METRIC, "value": b["batched"]["mpaths_s"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": 1, "ms_per_step": b["batched"]["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded batching configuration)",
            "config": {"workload": f"batching: {b['scenes']} sphere-union scenes (seed 100+i, edges 32-512 "
                                   f"log-uniform, occupancy U[10%,50%]), resolutions from {{128,256,512,1024}}^2, "
                                   f"Lambert 0.7, white sky, 4 bounces, {b['spp']} spp, one launch",
                       "paths_per_step": b["paths"], "voxels": b["voxels"]},
            "e2e": b.pop("e2e"), **b}


def serving_requests(rate: float, duration: float, seed: int = 3, pool_n: int = 16):
    """The seeded request stream: Poisson arrivals, sphere-union scenes (edge
    64-512) from a pool with reuse probability 0.5, random orbit cameras,
    resolution edge uniform in 256-1024, spp log-uniform in 16-1024."""
    from voxeltoy_gb300 import scenes as S
    rng = np.random.default_rng(seed)
    n = max(1, int(rng.poisson(rate * duration)))
    arrivals = np.sort(rng.uniform(0.0, duration, n))
    pool = []
    for i in range(pool_n):
        edge = int(rng.integers(64, 513))
        pool.append(S.sphere_union(edge, None, 300 + i, occupancy=float(rng.uniform(0.1, 0.5))))
    n_resident = 0
    reqs = []
    for k in range(n):
        res = int(rng.integers(256, 1025))
        spp = int(round(math.exp(rng.uniform(math.log(16), math.log(1024)))))
        reuse = n_resident > 0 and rng.random() < 0.5
        pick = int(rng.integers(0, n_resident)) if reuse else int(rng.integers(0, pool_n))
        cam = S.orbit_camera(distance=2000.0, theta_deg=float(rng.uniform(0, 360)), phi_deg=float(rng.uniform(10, 80)))
        reqs.append({"arrival": float(arrivals[k]), "res": res, "spp": spp, "reuse": reuse, "pick": pick, "cam": cam})
        if not reuse:
            n_resident += 1
    return reqs, pool


def serving_record(ctx, rate: float, duration: float, order: str = "arrival", quick_paths: int = 1 << 24,
                   round_cap: int = 0, alongside: bool = False, replay: bool = True, round_paths: int = 0) -> dict:
    """Config 4: the request stream served by vt_server (continuous batching)
    at its arrival times, then (replay) the same requests one at a time in
    arrival order in the plain form (the per-pixel kernel, one launch per
    pass: the reference's structure) and as one wavefront launch per request.
    Time-to-spp = arrival to the image being readable on the host; a replay's
    timeline is its measured service times queued behind one another from
    the same arrivals.  Every request's image is compared across the forms."""
    from voxeltoy_gb300 import Job, Scene, Server, scenes as S
    from voxeltoy_gb300 import _lib as L
    reqs, pool = serving_requests(rate, duration)
    settings = S.physical_settings(max_bounces=4, rr_start=-1, seed=0)
    srv = Server(ctx, hbm_budget_bytes=60 << 30, max_active_jobs=64, passes_per_round=4,
                 order=L.VT_SERVE_LEAST_WORK if order == "least-work" else L.VT_SERVE_ARRIVAL,
                 quick_paths=quick_paths, round_paths_cap=round_cap, round_paths=round_paths)
    scenes, scene_of, upload_s = [], [], {}
    large = big = None
    if alongside:
        # config 5 served alongside the stream: the voxelized icosphere at
        # 2048^2 x 1024 spp, 8 bounces, submitted when the stream starts
        v, f = S.fbm_displaced_icosphere(level=8)
        big = Scene.voxelize(ctx, np.ascontiguousarray(v, np.float32), np.ascontiguousarray(f, np.uint32),
                             (1024, 1024, 1024), mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE,
                             palette=[S.lambert(0.7)])
        bcfg = S.config1(edge=8, width=2048, height=2048, spp=1024)
        bcfg.settings.max_bounces = 8
    tickets = []
    pool_of = []            # the pool entry behind each resident scene index
    t_start = time.perf_counter()
    if alongside:
        large = srv.submit(big, None, bcfg.camera, bcfg.settings, 2048, 2048, 1024)
    for k, r in enumerate(reqs):
        wait = r["arrival"] - (time.perf_counter() - t_start)
        if wait > 0:
            time.sleep(wait)
        # the server keeps each volume resident under its key (the pool index);
        # a reused one is submitted without its voxels
        if r["reuse"]:
            si = r["pick"]
            vox = None
        else:
            pool_of.append(r["pick"])
            si = len(pool_of) - 1
            vox = pool[r["pick"]]
        scene_of.append(si)
        t0 = time.perf_counter()
        t = srv.submit_dense(si, vox, [S.lambert(0.7)], r["cam"], settings, r["res"], r["res"], r["spp"])
        t_ret = time.perf_counter()
        if vox is not None:
            upload_s[si] = t_ret - t0
        tickets.append((t, t_ret - t_start - r["arrival"]))
    lat, digests = [], []
    for (t, delay), r in zip(tickets, reqs):
        rc = srv.wait(t, 3600.0)
        if rc != 0:
            raise RuntimeError(f"request {t} failed: {rc}")
        img, secs = srv.result(t, r["res"], r["res"])
        lat.append(delay + secs)
        digests.append(image_digest(img))
    large_ms = None
    if large is not None:
        rc = srv.wait(large, 3600.0)
        if rc != 0:
            raise RuntimeError(f"the large request failed: {rc}")
        large_ms = srv_latency(srv, large) * 1e3
    t_end = time.perf_counter() - t_start
    stats = srv.stats()
    srv.close()
    # caller-owned copies of the scenes for the one-at-a-time replays
    scenes = [Scene.dense(ctx, pool[i], [S.lambert(0.7)]) for i in pool_of] if (replay and not alongside) else []
    paths = sum(r["res"] * r["res"] * r["spp"] for r in reqs) + (2048 * 2048 * 1024 if alongside else 0)
    lat = np.array(lat)
    rec = {"requests": len(reqs), "rate_req_s": rate, "duration_s": duration,
           "offered_mpaths_s": sum(r["res"] * r["res"] * r["spp"] for r in reqs) / duration / 1e6,
           "served": {"mpaths_s": paths / t_end / 1e6, "makespan_s": t_end,
                      "time_to_spp_ms": {"p50": float(np.percentile(lat, 50) * 1e3),
                                         "p99": float(np.percentile(lat, 99) * 1e3), "max": float(lat.max() * 1e3)},
                      "completed": int(stats.completed), "failed": int(stats.failed), "rounds": int(stats.rounds),
                      "scene_uploads": int(stats.scene_uploads), "scene_hits": int(stats.scene_hits),
                      "scene_evictions": int(stats.scene_evictions),
                      "round_s": stats.round_us / 1e6, "between_rounds_s": stats.between_us / 1e6},
           "settings": {"order": order, "quick_paths": quick_paths, "round_cap": round_cap,
                        "round_paths": round_paths or (1 << 26),
                        "hbm_budget_bytes": 60 << 30, "passes_per_round": 4, "max_active_jobs": 64,
                        "residency": "volumes kept resident by the server under their pool index "
                                     "(vt_server_submit_dense), uploaded at their first request"},
           "h2d_bytes": int(sum(pool[r["pick"]].nbytes for r in reqs if not r["reuse"]))}
    if alongside:
        rec["alongside"] = {"request": "voxelized icosphere (1.3M triangles, 1024^3) at 2048^2 x 1024 spp, 8 bounces, "
                                       "submitted with the first request of the stream", "time_to_spp_ms": large_ms}
    if replay and not alongside:
        same = True
        for name, kernel in (("plain", 1), ("per_request_wavefront", 2)):
            ctx.set_kernel(kernel)
            t_free, lats, busy = 0.0, [], 0.0
            first_use = set()
            for r, si, dg in zip(reqs, scene_of, digests):
                t0 = time.perf_counter()
                job = Job(ctx, scenes[si], None, r["cam"], settings, r["res"], r["res"])
                job.render(r["spp"])
                img = job.readback()
                dt = time.perf_counter() - t0
                job.close()
                if si not in first_use:     # the scene's upload, measured when it was served
                    first_use.add(si)
                    dt += upload_s.get(si, 0.0)
                start = max(r["arrival"], t_free)
                t_free = start + dt
                busy += dt
                lats.append(t_free - r["arrival"])
                same = same and image_digest(img) == dg
            lats = np.array(lats)
            rec[name] = {"mpaths_s": paths / t_free / 1e6, "makespan_s": t_free, "busy_s": busy,
                         "time_to_spp_ms": {"p50": float(np.percentile(lats, 50) * 1e3),
                                            "p99": float(np.percentile(lats, 99) * 1e3),
                                            "max": float(lats.max() * 1e3)}}
        ctx.set_kernel(2)
        rec["served_vs_plain"] = rec["plain"]["makespan_s"] / rec["served"]["makespan_s"]
        rec["served_vs_per_request_wavefront"] = rec["per_request_wavefront"]["makespan_s"] / rec["served"]["makespan_s"]
        rec["identical_images"] = bool(same)
    for sc in scenes:
        sc.close()
    if big is not None:
        big.close()
    return rec


def run_serving(args, world, rank, local):
    """Poisson request stream through vt_server (see serving_record)."""
    from voxeltoy_gb300 import Context
    ctx = Context(local)
    r = serving_record(ctx, args.rate, args.duration, order=args.order, quick_paths=args.quick_paths,
                       round_cap=args.round_cap, alongside=args.alongside, replay=args.replay,
                       round_paths=args.round_paths)
    ctx.close()
    s = r["served"]
    return {"metric": METRIC, "value": s["mpaths_s"], "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 0,
            "ms_per_step": s["makespan_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded request stream)",
            "config": {"workload": f"serving: Poisson {args.rate:g} req/s for {args.duration:g} s ({r['requests']} "
                                   f"requests), sphere-union scenes edge 64-512 (pool of 16), reuse 0.5, resolution "
                                   f"256^2-1024^2, 16-1024 spp log-uniform, 4 bounces, 60 GB admission budget, "
                                   f"admission order {args.order}, quick paths {args.quick_paths}, "
                                   f"round cap {args.round_cap}",
                       "requests": r["requests"], "offered_mpaths_s": r["offered_mpaths_s"]},
            "e2e": {"value": s["mpaths_s"], "unit": UNIT, "h2d_bytes_per_step": r["h2d_bytes"],
                    "d2h_bytes_per_step": 0}, **r}


def srv_latency(srv, ticket) -> float:
    """Submit-to-finish seconds of a finished request (the server's clock)."""
    import ctypes as C
    from voxeltoy_gb300 import _lib as L
    secs = C.c_double()
    L.call("vt_server_result", srv.h, ticket, None, 0, C.byref(secs))
    return secs.value


def config5_record(ctx, spp: int = 1024, steps: int = 3, check: bool = False, rmse_rows: int = 2) -> dict:
    """Config 5: the fBm-displaced icosphere (1,310,720 triangles) voxelized
    conservatively into 1024^3 (timed end to end, host mesh to resident
    scene), then rendered at 2048^2 x spp with config-1 materials and sky,
    8 bounces (CUDA events); relative RMSE of `rmse_rows` centre rows against
    the FP64 oracle, and optionally the occupancy against the oracle's."""
    import torch
    from voxeltoy_gb300 import Job, Scene, scenes as S
    from voxeltoy_gb300 import _lib as L
    v, f = S.fbm_displaced_icosphere(level=8)
    v = np.ascontiguousarray(v, np.float32)
    f = np.ascontiguousarray(f, np.uint32)
    res = (1024, 1024, 1024)
    vox_ms = []
    sc = None
    for k in range(steps + 1):
        if sc is not None:
            sc.close()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc = Scene.voxelize(ctx, v, f, res, mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE,
                            palette=[S.lambert(0.7)])
        sc.info()
        torch.cuda.synchronize()
        if k:
            vox_ms.append((time.perf_counter() - t0) * 1e3)
    cfg = S.config1(edge=8, width=2048, height=2048, spp=spp)
    cfg.settings.max_bounces = 8
    job = Job(ctx, sc, None, cfg.camera, cfg.settings, 2048, 2048)
    # the launch shape for this scene (its segments are longer than config 2's):
    # a short sweep at 64 spp per setting
    from voxeltoy_gb300 import autotune
    best = autotune.tune(ctx, [job], passes=64, repeats=1, use_cache=False,
                         grid={"path_slots": [1 << 25, 1 << 26], "trace_blocks_per_sm": [0], "trace_steps": [16, 32],
                               "lanes": [3], "brick_shape": [(2, 2, 2)], "queue_chunk": [128, 64],
                               "refill_min": [0], "trace_form_steps": []})
    tuning = {k: best[k] for k in ("path_slots", "trace_blocks_per_sm", "trace_steps", "lanes", "queue_chunk")}
    timer = EventTimer(ctx, ctx_device(ctx))
    job.render(4)
    job.reset()
    torch.cuda.synchronize()
    with timer:
        job.render(spp)
    paths = 2048 * 2048 * spp
    img = job.readback()
    job.close()
    cfg.voxels = sc.voxels()
    cfg.palette = [S.lambert(0.7)]
    sc.close()
    rec = {"triangles": int(len(f)), "grid": list(res), "spp": spp,
           "voxelize_ms": {"median": float(np.median(vox_ms)), "min": float(min(vox_ms))},
           "voxelize_mtris_s": len(f) / (np.median(vox_ms) * 1e-3) / 1e6,
           "render_ms": timer.ms, "render_mpaths_s": paths / (timer.ms * 1e-3) / 1e6,
           "image_finite": bool(np.isfinite(img).all()), "tuning": tuning}
    if rmse_rows > 0:
        r0 = (2048 - rmse_rows) // 2
        rec["rmse_vs_fp64"] = rmse_vs_fp64(cfg, img, spp, (r0, r0 + rmse_rows))
    if check:
        from oracle import binding as orc
        want = orc.voxelize(v, f, res, L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE)
        rec["occupancy_check"] = {"bit_exact": bool(np.array_equal(want, cfg.voxels)),
                                  "occupied": int(np.count_nonzero(cfg.voxels))}
    return rec


def config1_rmse(ctx) -> dict:
    """Config 1 at its full size (256^2 x 16 spp) against the FP64 oracle."""
    from voxeltoy_gb300 import Job, Scene, scenes as S
    cfg = S.config1()
    sc = Scene.dense(ctx, cfg.voxels, cfg.palette)
    job = Job(ctx, sc, None, cfg.camera, cfg.settings, cfg.width, cfg.height)
    job.render(cfg.spp)
    img = job.readback()
    job.close(); sc.close()
    return rmse_vs_fp64(cfg, img, cfg.spp, (0, cfg.height))


def converged_rmse(ctx, cfg, spp: int, emissive) -> dict:
    """The whole frame of `cfg` at `spp` samples per pixel (more than the
    benchmark frame's, so that the image is closer to converged) against the
    FP64 oracle at the same count.  The per-pixel difference comes from the
    few paths whose FP32 and FP64 arithmetic diverge, so it falls as
    1/sqrt(spp)."""
    from voxeltoy_gb300 import Env, Job, Scene
    sc = Scene.dense(ctx, cfg.voxels, cfg.palette, flags=cfg.scene_flags)
    env = Env(ctx, cfg.env_rgb) if cfg.env_rgb is not None else None
    job = Job(ctx, sc, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    job.render(spp)
    img = job.readback()
    for o in (job, env, sc):
        if o is not None:
            o.close()
    return rmse_vs_fp64(cfg, img, spp, (0, cfg.height), emissive=emissive)


def profile_voxelize(args, local):
    """--workload voxelize --profile: the config-5 scene (1024^3 from the
    1.3M-triangle mesh, voxelized 1 + --warmup times, each scene but the last
    closed) rendered at 2048^2 x --spp samples with the launch shape given on
    the command line, a frame per step, for ncu captures."""
    from voxeltoy_gb300 import Context, Job, Scene, scenes as S
    from voxeltoy_gb300 import _lib as L
    v, f = S.fbm_displaced_icosphere(level=8)
    ctx = Context(local)
    if args.slots > 0:
        ctx.set_lanes(args.lanes)
        ctx.set_tuning(args.slots, args.trace_bps, args.trace_steps)
    sc = None
    for k in range(1 + args.warmup):
        if sc is not None:
            sc.close()
        t0 = time.perf_counter()
        sc = Scene.voxelize(ctx, np.ascontiguousarray(v, np.float32), np.ascontiguousarray(f, np.uint32),
                            (1024, 1024, 1024), mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE,
                            palette=[S.lambert(0.7)])
        print(json.dumps({"voxelize_ms": 1e3 * (time.perf_counter() - t0)}), flush=True)
    cfg = S.config1(edge=8, width=2048, height=2048, spp=args.spp)
    cfg.settings.max_bounces = 8
    job = Job(ctx, sc, None, cfg.camera, cfg.settings, 2048, 2048)
    for k in range(args.warmup + args.steps):
        job.reset()
        t0 = time.perf_counter()
        job.render(args.spp)
        job.synchronize()
        if k >= args.warmup:
            print(json.dumps({"profile_step_ms": 1e3 * (time.perf_counter() - t0), "paths": 2048 * 2048 * args.spp,
                              "launches": ctx.launch_count()}), flush=True)
    job.close(); sc.close(); ctx.close()
    return 0


def run_voxelize(args, world, rank, local):
    """1.3M-triangle fBm-displaced icosphere, conservative voxelization into
    1024^3, then a 2048^2 render with config-1 materials and sky, 8 bounces."""
    from voxeltoy_gb300 import Context
    ctx = Context(local)
    spp = args.spp if args.spp != 256 else 1024
    r = config5_record(ctx, spp=spp, steps=args.steps, check=args.check, rmse_rows=2 if args.check else 0)
    ctx.close()
    return {"metric": METRIC, "value": r["render_mpaths_s"], "unit": UNIT, "n_gpus": world, "steps": 1,
            "warmup": 1, "ms_per_step": r["render_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded icosphere mesh)",
            "config": {"workload": f"voxelize: fBm-displaced icosphere level 8 ({r['triangles']} triangles) -> 1024^3 "
                                   f"conservative, then 2048^2 pinhole, Lambert 0.7, white sky, 8 bounces, {spp} spp",
                       "triangles": r["triangles"]},
            **r}


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
    ap.add_argument("--trace-form", type=int, default=-1, choices=[-1, 0, 1],
                    help="DDA kernel form with --slots: 0 per-lane set-up, 1 pooled set-up")
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
    ap.add_argument("--round-paths", type=int, default=0,
                    help="serving: paths traced per round (0 = the server's default, 2^26)")
    ap.add_argument("--alongside", action="store_true",
                    help="serving: also serve the voxelized 1.3M-triangle icosphere at 2048^2 x 1024 spp")
    ap.add_argument("--quick-paths", type=int, default=1 << 24,
                    help="serving: requests with at most this many paths left finish in one round (0 = off)")
    ap.add_argument("--check", action="store_true", help="voxelize: compare the occupancy with the oracle")
    ap.add_argument("--profile", action="store_true",
                    help="only warm-up and timed renders of the resident frame (for ncu captures)")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline line only: no RMSE check against the FP64 oracle and no batching, serving and "
                         "config-5 records")
    ap.add_argument("--extras-rate", type=float, default=16.0, help="request rate of the serving record")
    ap.add_argument("--extras-duration", type=float, default=5.0, help="seconds of arrivals of the serving record")
    ap.add_argument("--no-replay", dest="replay", action="store_false",
                    help="serving: skip the one-at-a-time replays of the stream")
    args = ap.parse_args()
    small = args.workload == "config1"
    args.edge = args.edge or (64 if small else 256)
    args.res = args.res or (256 if small else 1024)
    args.spp = args.spp or (16 if small else 256)
    args.steps = args.steps or (1000 if small and args.impl == "gb300" else 5)
    if args.impl == "gb300" and not args.profile:
        args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    extras = not args.no_extras and world == 1 and args.workload in ("config2", "config1")
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    from voxeltoy_gb300 import Context, Env, Job, Scene
    from voxeltoy_gb300 import _lib as L

    torch.cuda.set_device(local)
    if args.workload == "voxelize" and args.profile:
        return profile_voxelize(args, local)
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
        if args.trace_form >= 0:
            ctx.set_trace_form(args.trace_form)
        tuning = {"path_slots": args.slots, "trace_blocks_per_sm": args.trace_bps, "trace_steps": args.trace_steps,
                  "lanes": args.lanes, "trace_form": max(args.trace_form, 0), "source": "command line"}
    elif not args.no_tune and args.kernel == 2:
        from voxeltoy_gb300 import autotune
        best = autotune.tune(ctx, [job], passes=cfg.spp, repeats=1, use_cache=False)
        tuning = {k: best[k] for k in ("path_slots", "trace_blocks_per_sm", "trace_steps", "lanes", "trace_form",
                                       "queue_chunk", "refill_min", "brick_shape") if k in best}
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
    l2 = l2_read_gbs(ctx)
    frame_img = job.readback() if (rank == 0 and extras) else None   # the last timed frame, for the RMSE check

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
    issue = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text())
        if (t.get("workload") == args.workload and t.get("grid") == args.edge and t.get("res") == args.res
                and t.get("spp") == args.spp):
            traffic = t["dram_bytes_per_launch"]
            issue = t.get("dda_kernel")
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
                     "traffic_source": "profiles/traffic.json: small-case per-stream-position DRAM bytes scaled by the "
                                       "frame's stream positions",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "bytes_model": "1 B/DDA cell + 16 B/palette record + 8 B/env texel eval + 4 B/CDF probe + "
                                    "4 B/emissive read + 64 B/path framebuffer",
                     "l2": {"achieved": achieved, "peak": l2["gbs"], "unit": "GB/s", "frac": achieved / l2["gbs"],
                            "peak_source": l2["source"]},
                     # the DDA kernel (58% of the frame's kernel time) is bound by instruction issue and
                     # brick-load latency, not by bytes: its issue-slot utilisation from the committed profile
                     "issue": None if issue is None else
                     {"kernel": issue["kernel"], "achieved": issue["issue_active_pct"], "peak": issue["peak_issue_pct"],
                      "unit": "% of issue slots", "frac": issue["issue_active_pct"] / issue["peak_issue_pct"],
                      "warp_execution_efficiency_pct": issue["warp_execution_efficiency_pct"],
                      "thread_instructions_per_dda_cell": issue["thread_instructions_per_dda_cell"],
                      "source": issue["source"]}},
        "rates": {"gsegments_per_s": world * float(cnt[6]) / (ms * 1e-3) / 1e9,
                  "gdda_cells_per_s": world * float(cnt[1]) / (ms * 1e-3) / 1e9},
        "counters_per_frame": {"paths": int(cnt[0]), "dda_cells": int(cnt[1]), "palette": int(cnt[2]),
                               "env_evals": int(cnt[3]), "cdf_probes": int(cnt[4]), "emissive_reads": int(cnt[5]),
                               "segments": int(cnt[6]), "empty_brick_cells": int(cnt[7]),
                               "stream_positions": int(cnt[8])},
        "frame_ms": {"p50": float(np.percentile(times, 50)), "p99": float(np.percentile(times, 99)),
                     "note": "device time of each timed frame (one resident job from reset to its spp target)"},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "tuning": tuning,
    }
    emissive = scene.emissive()
    for o in (job, env, scene):
        if o is not None:
            o.close()
    if rank == 0 and extras:
        # checker and side records, outside every timed region above
        t_x = time.perf_counter()
        # the whole timed frame against the FP64 oracle at the same sample count
        rmse = {args.workload: rmse_vs_fp64(cfg, frame_img, cfg.spp, (0, cfg.height), emissive=emissive)}
        del frame_img
        if args.workload == "config2":
            rmse["config2_converged"] = converged_rmse(ctx, cfg, 4 * cfg.spp, emissive)
            rmse["config1"] = config1_rmse(ctx)
            b = batching_record(ctx, args.scenes, 3, e2e=False)
            rmse["config3"] = b.pop("rmse_vs_fp64")
            c5 = config5_record(ctx, spp=1024, steps=2, rmse_rows=2)
            rmse["config5"] = c5.pop("rmse_vs_fp64")
            srv = serving_record(ctx, args.extras_rate, args.extras_duration)
            line["batching"] = b
            line["serving"] = srv
            line["config5"] = c5
            line["batched_vs_plain"] = b["batched_vs_plain"]
            line["served_vs_plain"] = srv["served_vs_plain"]
            line["time_to_spp_ms"] = dict(srv["served"]["time_to_spp_ms"],
                                          stream=f"Poisson {args.extras_rate:g} req/s for {args.extras_duration:g} s")
        line["rmse_vs_fp64"] = rmse
        recs = [r for v in rmse.values() for r in (v if isinstance(v, list) else [v])]
        line["rmse_max"] = max(r["rel_rmse"] for r in recs)
        line["extras_s"] = round(time.perf_counter() - t_x, 1)
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
