"""Autotuner of the wavefront renderer's launch parameters.

Times short renders of the caller's own jobs over a grid of
  path_slots            paths in flight per launch (state + queues per slot)
  trace_blocks_per_sm   resident blocks of the DDA kernel (rays per block x
                        blocks: the DDA kernel's block shape is 256 threads)
  trace_steps           DDA steps between ray-pool refills
  lanes                 wavefronts side by side on as many streams (1-3)
and then, at the best of those, a second sweep of
  brick_shape           log2 extents of the scenes' occupancy bricks (4x4x4,
                        8x4x2, 2x8x4, 4x2x8: 64 voxels a word)
  queue_chunk           queue records a DDA warp takes per atomic
  refill_min            compaction threshold: a DDA warp refills its lanes as
                        soon as fewer than this many still step (0 = only
                        every trace_steps steps)
and last the pooled form of the DDA kernel (segment set-up for a warp's
worth of records at once, lanes refilled from a shared-memory pool) at
trace_form_steps steps per batch.
and applies the fastest setting to the context.  Every setting renders the
same bits.  Path-slot counts above the workload's samples collapse to one
setting; frames shorter than a few milliseconds are timed several times per
setting.  Results are cached in a JSON file keyed by a workload class (log2
of the largest grid edge, log2 of the pixels per pass, number of jobs) and
the set of knobs swept, so later runs with a similar workload skip the sweep.
"""
from __future__ import annotations

import itertools
import json
import math
import os
import time
from pathlib import Path

DEFAULT_GRID = {
    "path_slots": [1 << 22, 1 << 23, 1 << 24, 1 << 25],
    "trace_blocks_per_sm": [0, 3, 5],
    "trace_steps": [8, 16, 32],
    "lanes": [2, 3, 1],
    "brick_shape": [(2, 2, 2), (3, 2, 1), (1, 3, 2), (2, 1, 3)],
    "queue_chunk": [128, 64, 256],
    "refill_min": [0, 12, 20],
    "trace_form_steps": [8, 16],
}
KNOBS = "slots,bps,steps,lanes,brick,chunk,refill,form"


def cache_path() -> Path:
    base = os.environ.get("VOXELTOY_TUNE_CACHE")
    if base:
        return Path(base)
    return Path.home() / ".cache" / "voxeltoy_gb300" / "tune.json"


def workload_key(jobs) -> str:
    edge = max(max(j.scene.info().resolution) for j in jobs)
    pixels = sum(j.width * j.height for j in jobs)
    return (f"edge{int(round(math.log2(max(edge, 1))))}_px{int(round(math.log2(max(pixels, 1))))}_jobs{len(jobs)}"
            f"_{KNOBS}")


def _apply(ctx, setting: dict, jobs=()):
    ctx.set_lanes(setting.get("lanes", 2))
    ctx.set_tuning(setting["path_slots"], setting["trace_blocks_per_sm"], setting["trace_steps"])
    ctx.set_trace_tuning(setting.get("queue_chunk", 128), setting.get("refill_min", 0))
    if hasattr(ctx, "set_trace_form"):
        ctx.set_trace_form(setting.get("trace_form", 0))
    shape = tuple(setting.get("brick_shape", (2, 2, 2)))
    for sc in {id(j.scene): j.scene for j in jobs}.values():
        if tuple(sc.brick_shape()) != shape:
            sc.set_brick_shape(shape)


def _time_render(ctx, jobs, passes: int, repeats: int) -> float:
    best = float("inf")
    for _ in range(repeats):
        for j in jobs:
            j.reset()
        for j in jobs:
            j.synchronize()
        t0 = time.perf_counter()
        if len(jobs) == 1:
            jobs[0].render(passes)
        else:
            ctx.render_batch(jobs, passes)
        for j in jobs:
            j.synchronize()
        best = min(best, time.perf_counter() - t0)
    return best


def tune(ctx, jobs, passes: int = 16, repeats: int = 2, grid: dict | None = None, use_cache: bool = True) -> dict:
    """Sweep the grid on `passes` samples per pixel of `jobs`, apply and return
    the best setting ({"path_slots", "trace_blocks_per_sm", "trace_steps",
    "lanes", "seconds", "key", "cached"}).  `grid` overrides entries of
    DEFAULT_GRID."""
    key = workload_key(jobs)
    path = cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        best = dict(cache[key])
        _apply(ctx, best, jobs)
        best.update(key=key, cached=True)
        return best
    grid = dict(DEFAULT_GRID, **(grid or {}))
    items = passes * sum(j.width * j.height for j in jobs)
    slot_list = sorted({min(s, max(items, 32)) for s in grid["path_slots"]})
    _apply(ctx, {"path_slots": slot_list[-1], "trace_blocks_per_sm": 0, "trace_steps": 16})
    _time_render(ctx, jobs, passes, 1)                                   # warm: buffers, graphs
    once = _time_render(ctx, jobs, passes, 1)
    reps = max(repeats, min(50, math.ceil(0.03 / max(once, 1e-6))))
    results = []
    for lanes, slots, bps, steps in itertools.product(grid["lanes"], slot_list, grid["trace_blocks_per_sm"],
                                                      grid["trace_steps"]):
        setting = {"path_slots": slots, "trace_blocks_per_sm": bps, "trace_steps": steps, "lanes": lanes,
                   "brick_shape": tuple(grid["brick_shape"][0]), "queue_chunk": grid["queue_chunk"][0],
                   "refill_min": grid["refill_min"][0], "trace_form": 0}
        _apply(ctx, setting, jobs)
        results.append((_time_render(ctx, jobs, passes, reps), setting))
    results.sort(key=lambda r: r[0])
    # the bricks and the DDA kernel's queue chunk and compaction threshold at
    # the best launch shape
    first = dict(results[0][1])
    for shape, chunk, refill in itertools.product(grid["brick_shape"], grid["queue_chunk"], grid["refill_min"]):
        if (tuple(shape), chunk, refill) == (first["brick_shape"], first["queue_chunk"], first["refill_min"]):
            continue
        setting = dict(first, brick_shape=tuple(shape), queue_chunk=chunk, refill_min=refill)
        _apply(ctx, setting, jobs)
        results.append((_time_render(ctx, jobs, passes, reps), setting))
    results.sort(key=lambda r: r[0])
    # the pooled DDA form at the best setting so far (the compaction threshold does not apply to it)
    second = dict(results[0][1])
    for steps in grid.get("trace_form_steps", []):
        setting = dict(second, trace_form=1, trace_steps=steps, refill_min=0)
        _apply(ctx, setting, jobs)
        results.append((_time_render(ctx, jobs, passes, reps), setting))
    results.sort(key=lambda r: r[0])
    # the three fastest settings again, three times as long each: single
    # timings a fraction of a percent apart do not pick a winner reliably
    final = []
    for _, setting in results[:3]:
        _apply(ctx, setting, jobs)
        final.append((_time_render(ctx, jobs, passes, 3 * reps), setting))
    final.sort(key=lambda r: r[0])
    t, best = final[0]
    _apply(ctx, best, jobs)
    best = dict(best, seconds=t)
    for j in jobs:
        j.reset()
    if use_cache:
        cache[key] = best
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    best.update(key=key, cached=False, repeats=reps, sweep=[dict(r[1], seconds=r[0]) for r in results])
    return best
