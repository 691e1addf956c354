"""vt_render_batch_fixed: the wavefront renderer on the library's fixed device
array.  Called through the C ABI and compared with vt_render_batch (the same
kernels on context-allocated buffers), bit for bit, on two calls in a row.
The file name puts it last in collection so that it also runs after every
other GPU test has used the device; it creates its own context and passes
alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

from helpers import close_all, gpu_setup, small_config1, small_config2
from voxeltoy_gb300 import Context, Job
from voxeltoy_gb300 import _lib as L

pytestmark = pytest.mark.gpu

MAX_JOBS, MAX_SLOTS, MAX_SAMPLES = 16, 65536, 1 << 20


@pytest.fixture(scope="module")
def fctx():
    c = Context()
    yield c
    c.close()


def fixed(ctx, jobs, passes, path_slots=0):
    """vt_render_batch_fixed through ctypes; returns (status, results)."""
    lib = L.load()
    arr = (C.c_void_p * max(1, len(jobs)))(*[j.h.value for j in jobs])
    res = (C.c_int32 * max(1, len(jobs)))()
    rc = lib.vt_render_batch_fixed(ctx.h, arr, len(jobs), passes, path_slots, res)
    return rc, list(res)[: len(jobs)]


def bits(job):
    return job.readback().view(np.uint32).copy()


def device_free_bytes() -> int:
    import torch
    return torch.cuda.mem_get_info()[0]


def test_fixed_equals_batch_and_allocates_nothing(fctx):
    cfg = small_config2(edge=32, w=40, h=28, seed=11)
    cfg.settings.max_samples = 1 << 20
    scene, env, ref = gpu_setup(fctx, cfg)
    job = Job(fctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    try:
        for call in range(2):                       # two calls in a row
            before = fctx.memory()
            free_before = device_free_bytes()
            rc, res = fixed(fctx, [job], 3)
            assert rc == L.VT_OK, L.load().vt_last_error()
            assert fctx.memory() == before          # nothing drawn from the context's allocator
            if call == 1:
                # nor from the device: the array was reserved when the context
                # was created (the first call may still load kernel code)
                assert device_free_bytes() == free_before
            assert res == [L.VT_SAMPLES_PENDING]
            fctx.render_batch([ref], 3, kernel=2)
            assert job.samples() == ref.samples() == 3 * (call + 1)
            np.testing.assert_array_equal(bits(job), bits(ref))
    finally:
        close_all(job, ref, scene, env)


def test_fixed_batches_split_over_launches(fctx):
    """Two jobs whose samples exceed one launch's sample buffer, a small
    path-slot count and a sample cap that stops one job mid-call."""
    cfgs = [small_config1(edge=40, w=64, h=48, seed=12), small_config2(edge=32, w=40, h=40, seed=13)]
    cfgs[0].settings.max_samples = 1 << 20
    cfgs[1].settings.max_samples = 250
    made = [gpu_setup(fctx, c) for c in cfgs]
    refs = [Job(fctx, s, e, c.camera, c.settings, c.width, c.height) for (s, e, _j), c in zip(made, cfgs)]
    jobs = [m[2] for m in made]
    passes = 2 * MAX_SAMPLES // (64 * 48 + 40 * 40) // 3 * 2      # more than fits in one launch
    try:
        for call in range(2):
            rc, res = fixed(fctx, jobs, passes, path_slots=4096)
            assert rc == L.VT_OK, L.load().vt_last_error()
            want = fctx.render_batch(refs, passes, kernel=2)
            assert res == want
            for j, r in zip(jobs, refs):
                assert j.samples() == r.samples()
                np.testing.assert_array_equal(bits(j), bits(r))
        assert jobs[1].samples() == 250 and res[1] == L.VT_FINISHED_RENDERING
    finally:
        close_all(*refs)
        for s, e, j in made:
            close_all(j, s, e)


def test_fixed_rejects_sizes_beyond_its_limits(fctx):
    lib = L.load()
    cfg = small_config1(edge=24, w=16, h=16, seed=14)
    scene, env, job = gpu_setup(fctx, cfg)
    big = Job(fctx, scene, env, cfg.camera, cfg.settings, 1025, 1024)
    try:
        rc, _ = fixed(fctx, [job] * (MAX_JOBS + 1), 1)
        assert rc == L.VT_EINVAL and b"VT_FIXED_MAX_JOBS" in lib.vt_last_error()
        rc, _ = fixed(fctx, [job], 1, path_slots=MAX_SLOTS + 1)
        assert rc == L.VT_EINVAL and b"VT_FIXED_MAX_PATH_SLOTS" in lib.vt_last_error()
        rc, _ = fixed(fctx, [job, big], 1)
        assert rc == L.VT_EINVAL and b"VT_FIXED_MAX_SAMPLES" in lib.vt_last_error()
        assert job.samples() == 0 and big.samples() == 0
        rc, _ = fixed(fctx, [job], 1, path_slots=MAX_SLOTS)
        assert rc == L.VT_OK and job.samples() == 1
    finally:
        close_all(big, job, scene, env)
