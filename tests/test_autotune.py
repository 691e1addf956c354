"""The autotuner's sweep logic on the CPU, against fake jobs whose render time
depends on the setting applied to a fake context."""
import json

import pytest

from voxeltoy_gb300 import autotune


class FakeInfo:
    def __init__(self, res):
        self.resolution = res


class FakeScene:
    def __init__(self, res, ctx=None):
        self._res = res
        self.ctx = ctx
        self.shape = (2, 2, 2)

    def info(self):
        return FakeInfo(self._res)

    def brick_shape(self):
        return self.shape

    def set_brick_shape(self, shape):
        self.shape = tuple(shape)
        if self.ctx is not None:
            self.ctx.setting["brick_shape"] = self.shape


class FakeCtx:
    def __init__(self):
        self.setting = {}
        self.applied = []

    def set_tuning(self, slots, bps, steps):
        self.setting.update(path_slots=slots, trace_blocks_per_sm=bps, trace_steps=steps)
        self.applied.append(dict(self.setting))

    def set_lanes(self, lanes):
        self.setting["lanes"] = lanes

    def set_trace_tuning(self, queue_chunk, refill_min):
        self.setting.update(queue_chunk=queue_chunk, refill_min=refill_min)

    def set_trace_form(self, form):
        self.setting["trace_form"] = form

    def render_batch(self, jobs, passes):
        for j in jobs:
            j.render(passes)


class FakeJob:
    """Render 'time' is spent in a fake clock: the best setting is 8M slots,
    3 blocks per SM, 16 steps, two lanes, 8x4x2 bricks, queue chunks of 64
    and a refill threshold of 12."""

    def __init__(self, ctx, clock, w=64, h=48, res=(32, 32, 32), unit=1.0):
        self.ctx, self.clock, self.unit = ctx, clock, unit
        self.width, self.height = w, h
        self.scene = FakeScene(res, ctx)
        self.renders = 0

    def reset(self):
        pass

    def synchronize(self):
        pass

    def render(self, passes):
        s = self.ctx.setting
        cost = 1.0
        cost += 0.1 * abs(s.get("path_slots", 0) - (1 << 23)) / (1 << 23)
        cost += 0.05 * abs(s.get("trace_blocks_per_sm", 0) - 3)
        cost += 0.03 * abs(s.get("trace_steps", 16) - 16) / 8
        cost += 0.07 * abs(s.get("lanes", 2) - 2)
        cost += 0.01 * abs(s.get("queue_chunk", 128) - 64) / 64
        cost += 0.002 * abs(s.get("refill_min", 0) - 12)
        cost += 0.0 if self.scene.shape == (3, 2, 1) else 0.004
        cost += 0.05 * s.get("trace_form", 0)
        self.clock[0] += cost * passes * self.unit
        self.renders += 1


@pytest.fixture
def fake_time(monkeypatch):
    clock = [0.0]
    monkeypatch.setattr(autotune.time, "perf_counter", lambda: clock[0])
    return clock


def test_sweep_picks_the_fastest_setting(fake_time, tmp_path, monkeypatch):
    monkeypatch.setenv("VOXELTOY_TUNE_CACHE", str(tmp_path / "tune.json"))
    ctx = FakeCtx()
    job = FakeJob(ctx, fake_time, w=4096, h=4096)    # enough samples that no slot count collapses
    best = autotune.tune(ctx, [job], passes=16, repeats=1, use_cache=False)
    assert (best["path_slots"], best["trace_blocks_per_sm"], best["trace_steps"], best["lanes"],
            best["brick_shape"], best["queue_chunk"], best["refill_min"]) == (1 << 23, 3, 16, 2, (3, 2, 1), 64, 12)
    assert ctx.setting == {"path_slots": 1 << 23, "trace_blocks_per_sm": 3, "trace_steps": 16, "lanes": 2,
                           "brick_shape": (3, 2, 1), "queue_chunk": 64, "refill_min": 12, "trace_form": 0}
    assert best["trace_form"] == 0
    assert job.scene.shape == (3, 2, 1)
    g = autotune.DEFAULT_GRID
    # the launch-shape grid, then bricks and the DDA kernel's knobs at the best launch shape, then the pooled form
    assert len(best["sweep"]) == len(g["path_slots"]) * len(g["trace_blocks_per_sm"]) * len(g["trace_steps"]) * \
        len(g["lanes"]) + len(g["brick_shape"]) * len(g["queue_chunk"]) * len(g["refill_min"]) - 1 + \
        len(g["trace_form_steps"])
    assert not (tmp_path / "tune.json").exists()


def test_slot_counts_collapse_to_the_frame_and_short_frames_repeat(fake_time):
    ctx = FakeCtx()
    job = FakeJob(ctx, fake_time, w=16, h=16, unit=1e-4)   # 16 x 16 x 4 = 1024 samples, 0.4 ms a frame
    best = autotune.tune(ctx, [job], passes=4, repeats=1, use_cache=False)
    assert {r["path_slots"] for r in best["sweep"]} == {1024}
    assert best["repeats"] == 50                     # a frame far below 30 ms is timed up to 50 times


def test_cache_round_trip(fake_time, tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("VOXELTOY_TUNE_CACHE", str(path))
    ctx = FakeCtx()
    job = FakeJob(ctx, fake_time, w=4096, h=4096)
    first = autotune.tune(ctx, [job], passes=16, repeats=1, grid={"path_slots": [1 << 22, 1 << 23]})
    assert first["cached"] is False and path.exists()
    key = autotune.workload_key([job])
    assert json.loads(path.read_text())[key]["path_slots"] == 1 << 23
    ctx2 = FakeCtx()
    job2 = FakeJob(ctx2, fake_time, w=4096, h=4096)
    second = autotune.tune(ctx2, [job2], passes=16, repeats=1)
    assert second["cached"] is True and job2.renders == 0
    assert ctx2.setting["path_slots"] == 1 << 23 and ctx2.setting["lanes"] == first["lanes"]


def test_workload_key_classes():
    ctx, clock = FakeCtx(), [0.0]
    a = FakeJob(ctx, clock, w=512, h=512, res=(256, 256, 256))
    b = FakeJob(ctx, clock, w=500, h=520, res=(250, 240, 260))
    c = FakeJob(ctx, clock, w=512, h=512, res=(1024, 64, 64))
    assert autotune.workload_key([a]) == autotune.workload_key([b])
    assert autotune.workload_key([a]) != autotune.workload_key([c])
    assert "_jobs2_" in autotune.workload_key([a, b])
    assert autotune.workload_key([a]).endswith(autotune.KNOBS)     # entries of an older knob set do not apply
