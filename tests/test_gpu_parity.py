"""GPU parity: the CUDA kernels against the CPU restatement of the reference.

Bit-exact for everything integer or index valued (DDA hits and faces,
voxelizer occupancy, emissive lists) and, because both sides evaluate the
same IEEE single-precision operations, for per-sample radiance too.  The
converged image is compared with the FP64 oracle by relative RMSE <= 1e-3.
"""
import math
import time

import numpy as np
import pytest

from helpers import (bricks_from_voxels, close_all, gpu_setup, oracle_setup, reference_config, small_config1,
                     small_config2)
from voxeltoy_gb300 import Env, Job, Scene, Server
from voxeltoy_gb300 import _lib as L
from voxeltoy_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    """Bitwise float equality, any NaN equal to any NaN (NaN payloads differ
    between the GPU and the host C library)."""
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


def test_builtins_bitexact(ctx, orc):
    rng = np.random.default_rng(0)
    a = np.concatenate([rng.uniform(-30, 30, 100000), rng.uniform(-1, 1, 50000)]).astype(np.float32)
    b = rng.uniform(0.01, 800, a.size).astype(np.float32)
    pos = np.abs(a) + np.float32(1e-7)
    for fn, x, y in [(0, a, None), (1, a, None), (2, pos, b), (3, np.clip(a, -1, 1), None), (4, a, b),
                     (5, pos, None), (6, a * 4, None), (7, a * 1000, None)]:
        got = ctx.builtins(fn, x, y)
        want = orc.builtins(fn, x, y)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=f"fn {fn}")


def _rays(rng, n):
    """Half the rays start at the volume's entry point of a ray from a shell
    around it (as the integrator clips primary rays, pathTracer.fs:183-196),
    half start at random points inside the volume."""
    d0 = rng.normal(size=(n, 3))
    d0 /= np.linalg.norm(d0, axis=1, keepdims=True)
    far = -1500.0 * d0
    targets = rng.uniform(-450, 450, (n, 3))
    dirs = targets - far
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    with np.errstate(divide="ignore"):
        t0 = (-500.0 - far) / dirs
        t1 = (500.0 - far) / dirs
    tmin = np.minimum(t0, t1).max(axis=1)
    origins = far + tmin[:, None] * dirs
    inside = rng.uniform(-499, 499, (n, 3))
    half = n // 2
    origins[half:] = inside[half:]
    return origins.astype(np.float32), dirs.astype(np.float32)


def _special_rays():
    o, d = [], []
    for axis in range(3):
        for s in (-1.0, 1.0):
            v = np.zeros(3); v[axis] = s
            o.append(-v * 900 + np.array([3.3, 7.1, -5.5])); d.append(v)
    for dd in [(1, 1, 1), (-1, 1, -1), (1, -1, 0), (0, 1, 1)]:
        v = np.array(dd, float); v /= np.linalg.norm(v)
        o.append(-v * 900); d.append(v)
    for eps in (1e-6, -1e-6, 5e-6):                       # grazing components
        v = np.array([1.0, eps, 0.3]); o.append([-800, 12.0, 1.0]); d.append(v / np.linalg.norm(v))
    o.append([0.0, 0.0, 0.0]); d.append([0.0, -1.0, 0.0])  # inside the volume
    o.append([15.625, 100.0, 31.25]); d.append([0.0, 1.0, 0.0])  # on voxel faces
    o.append([600.0, 600.0, 600.0]); d.append([1.0, 0.0, 0.0])   # outside, pointing away
    return np.array(o, np.float32), np.array(d, np.float32)


@pytest.mark.parametrize("quirks", [0, L.VT_QUIRK_GROUND])
def test_trace_rays_bitexact(ctx, orc, quirks):
    cfg = small_config1(edge=64)
    cfg.settings.quirks = quirks
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        rng = np.random.default_rng(11)
        o, d = _rays(rng, 200000)
        so, sd = _special_rays()
        o = np.concatenate([o, so]); d = np.concatenate([d, sd])
        got = job.trace_rays(o, d)
        want = orc.trace_rays(orc.Scene(cfg.voxels, cfg.palette), o, d, quirks)
        np.testing.assert_array_equal(got, want)
        hits = (got[:, 3] >> 8) & 1
        assert 0.2 < hits.mean() < 0.95
    finally:
        close_all(job, scene, env)


def test_env_build_bitexact(ctx, orc):
    rgb = S.sky_sun_env(96, 48)
    rgb[3, 5] = 70000.0   # beyond half range: stored as infinity in both
    rgb[10, 40] = [0.0, 0.0, 0.0]
    env = Env(ctx, np.ascontiguousarray(rgb))
    try:
        cu, cv, integral = env.cdf()
        ref = orc.Env(rgb, chunk=32)
        np.testing.assert_array_equal(env.texels(), ref.texels)
        np.testing.assert_array_equal(cu, ref.cdf_u)
        np.testing.assert_array_equal(cv, ref.cdf_v)
        assert integral == np.float32(ref.integral)
        seq = orc.Env(rgb, chunk=0)   # strictly sequential FP64 sums: within one float ulp
        assert np.all(np.abs(cu - seq.cdf_u) <= np.spacing(np.float32(1.0)))
    finally:
        env.close()


@pytest.mark.parametrize("size", [(1100, 550), (777, 333), (300, 900)])
def test_env_reference_size_cdf_bitexact(ctx, orc, size):
    """VT_ENV_CDF_REFERENCE_SIZE: full-size texels, CDFs and integral of the
    image shrunk to at most 512 texels on its long axis, equal to the
    oracle's build of the same mode bit for bit."""
    w, h = size
    rgb = np.ascontiguousarray(S.sky_sun_env(w, h, peak=300.0))
    env = Env(ctx, rgb, flags=L.VT_ENV_CDF_REFERENCE_SIZE)
    try:
        ref = orc.Env(rgb, chunk=32, flags=1)
        assert (env.cdf_w, env.cdf_h) == orc.cdf_size(w, h)
        assert max(env.cdf_w, env.cdf_h) == 512
        cu, cv, integral = env.cdf()
        np.testing.assert_array_equal(env.texels(), ref.texels)
        np.testing.assert_array_equal(cu, ref.cdf_u)
        np.testing.assert_array_equal(cv, ref.cdf_v)
        assert integral == np.float32(ref.integral)
    finally:
        env.close()


def test_samples_bitexact_reference_size_env(ctx, orc):
    """Per-sample radiance and first hits with importance sampling through
    the shrunk CDFs (pdf from the full-size texels) equal the oracle's."""
    cfg = small_config2(edge=32, w=32, h=28, seed=5)
    cfg.env_rgb = S.sky_sun_env(1040, 520, peak=400.0)
    scene = Scene.dense(ctx, cfg.voxels, cfg.palette, flags=cfg.scene_flags)
    env = Env(ctx, cfg.env_rgb, flags=L.VT_ENV_CDF_REFERENCE_SIZE)
    job = Job(ctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    try:
        assert (env.cdf_w, env.cdf_h) == (512, 256)
        osc = orc.Scene(cfg.voxels, cfg.palette, scene.emissive())
        oenv = orc.Env(cfg.env_rgb, flags=1)
        for smp in (0, 3):
            g_rgba, g_hits, g_cnt = job.samples_diag(smp)
            o_rgba, o_hits, o_cnt = orc.render_samples(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height,
                                                       smp, 32)
            np.testing.assert_array_equal(g_hits, o_hits)
            assert same_bits(g_rgba, o_rgba).all()
            assert g_cnt[4] > 0                      # the CDFs were probed
    finally:
        close_all(job, scene, env)


def test_gpu_cdf_known_answers(ctx):
    cu, cv, _ = ctx.cdf_from_function(np.array([[1, 1, 0, 2, 1, 0, 5], [2, 1, 5, 0, 0, 1, 3],
                                                [128, 0, 0, 0, 0, 0, 0]], np.float32))
    assert cu[0].tolist() == [np.float32(x) for x in (0, 0.1, 0.2, 0.2, 0.4, 0.5, 0.5, 1.0)]
    np.testing.assert_array_equal(cv, np.float32([0, 10 / 150, 22 / 150, 1]))


def _compare_samples(ctx, orc, cfg, samples=(0, 1, 2), noise=False):
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        osc, oenv = oracle_setup(orc, cfg, scene, env)
        table = ctx.noise_table() if noise else None
        for smp in samples:
            g_rgba, g_hits, g_cnt = job.samples_diag(smp)
            o_rgba, o_hits, o_cnt = orc.render_samples(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height,
                                                       smp, 32, noise=table)
            np.testing.assert_array_equal(g_hits, o_hits, err_msg=f"first hits, sample {smp}")
            bad = np.argwhere(~same_bits(g_rgba, o_rgba))
            assert bad.size == 0, f"sample {smp}: {len(bad)} values differ, first {bad[:4].tolist()}"
            np.testing.assert_array_equal(g_cnt[:7], o_cnt[:7])
        return g_rgba
    finally:
        close_all(job, scene, env)


def test_samples_bitexact_config1(ctx, orc):
    img = _compare_samples(ctx, orc, small_config1())
    assert np.isfinite(img).all() and img[..., :3].max() > 0.1


def test_samples_bitexact_config2(ctx, orc):
    cfg = small_config2()
    img = _compare_samples(ctx, orc, cfg, samples=(0, 5))
    assert np.isfinite(img).all()


def test_samples_bitexact_reference_quirks(ctx, orc):
    cfg = reference_config()
    _compare_samples(ctx, orc, cfg, samples=(0, 3), noise=True)


def test_samples_bitexact_reference_quirks_image_env(ctx, orc):
    cfg = reference_config(seed=4)
    cfg.env_rgb = S.sky_sun_env(48, 24, peak=200.0)
    cfg.settings.background_rotation = 0.7
    _compare_samples(ctx, orc, cfg, samples=(1,), noise=True)


def test_samples_bitexact_ortho_wireframe_selection(ctx, orc):
    cfg = small_config1(edge=32, w=33, h=29)
    cfg.camera.lens_model = L.VT_LENS_ORTHOGRAPHIC
    cfg.settings.wireframe_opacity = 0.6
    cfg.settings.wireframe_thickness = 0.05
    occ = np.argwhere(cfg.voxels > 0)
    z, y, x = occ[len(occ) // 2]
    cfg.settings.selected_voxel[:] = [int(x), int(y), int(z)]
    cfg.settings.select_enabled = 1
    _compare_samples(ctx, orc, cfg, samples=(0, 1))


def _compare_edit_samples(ctx, orc, cfg, samples=(0, 1), noise=False):
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        job.set_integrator(L.VT_INTEGRATOR_EDIT_MODE)
        osc, oenv = oracle_setup(orc, cfg, scene, env)
        table = ctx.noise_table() if noise else None
        for smp in samples:
            g_rgba, g_hits, g_cnt = job.samples_diag(smp)
            o_rgba, o_hits, o_cnt = orc.render_samples(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height,
                                                       smp, 32, noise=table, integrator=1)
            np.testing.assert_array_equal(g_hits, o_hits, err_msg=f"first hits, sample {smp}")
            np.testing.assert_array_equal(g_rgba.view(np.uint32), o_rgba.view(np.uint32), err_msg=f"sample {smp}")
            np.testing.assert_array_equal(g_cnt[:7], o_cnt[:7])
        return g_rgba
    finally:
        close_all(job, scene, env)


def test_edit_mode_samples_bitexact(ctx, orc):
    """editMode.fs on the GPU against the oracle: selection and wireframe,
    an environment background, and the reference's quirks (ground hits,
    noise-table random numbers)."""
    cfg = small_config1(edge=32, w=33, h=29, seed=21)
    cfg.settings.wireframe_opacity = 0.6
    cfg.settings.wireframe_thickness = 0.05
    occ = np.argwhere(cfg.voxels > 0)
    z, y, x = occ[len(occ) // 3]
    cfg.settings.selected_voxel[:] = [int(x), int(y), int(z)]
    cfg.settings.select_enabled = 1
    img = _compare_edit_samples(ctx, orc, cfg)
    assert np.isfinite(img).all() and img[..., :3].max() > 0
    _compare_edit_samples(ctx, orc, small_config2(edge=40, w=36, h=28, seed=22), samples=(0,))
    _compare_edit_samples(ctx, orc, reference_config(seed=23), samples=(0, 2), noise=True)


def test_edit_mode_accumulation_and_switch(ctx, orc):
    """Edit-mode passes through vt_job_render and vt_render_batch_fixed
    accumulate like the oracle's running average; a switch restarts the
    accumulation."""
    import ctypes as C
    cfg = small_config2(edge=32, w=30, h=22, seed=24)
    scene, env, job = gpu_setup(ctx, cfg)
    other = Job(ctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    try:
        job.render(2)
        assert job.samples() == 2
        job.set_integrator(L.VT_INTEGRATOR_EDIT_MODE)
        assert job.samples() == 0
        job.render(3)
        got = job.readback()
        osc, oenv = oracle_setup(orc, cfg, scene, env)
        want, _ = orc.render_average(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, 3, 32, integrator=1)
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
        other.set_integrator(L.VT_INTEGRATOR_EDIT_MODE)
        arr = (C.c_void_p * 1)(other.h.value)
        res = (C.c_int32 * 1)()
        assert L.load().vt_render_batch_fixed(ctx.h, arr, 1, 3, 0, res) == L.VT_OK
        np.testing.assert_array_equal(other.readback().view(np.uint32), got.view(np.uint32))
        job.set_integrator(L.VT_INTEGRATOR_PATH_TRACER)
        assert job.samples() == 0
        with pytest.raises(L.VtError):
            job.set_integrator(2)
    finally:
        close_all(other, job, scene, env)


def _plain_equals_wavefront(ctx, cfg, passes=3):
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        ctx.set_kernel(1)
        job.render(passes)
        a = job.readback().copy()
        job.reset()
        ctx.set_kernel(2)
        job.render(passes)
        np.testing.assert_array_equal(a.view(np.uint32), job.readback().view(np.uint32))
    finally:
        ctx.set_kernel(2)
        close_all(job, scene, env)


@pytest.mark.parametrize("shape", [(23, 37, 50), (5, 64, 9), (61, 7, 30)])
def test_ragged_volume_bitexact(ctx, orc, shape):
    """Volumes whose sides differ and are not multiples of the 4-voxel brick:
    the partial border bricks, the world bounds on the major axis and the
    emissive list of a cropped grid."""
    cfg = small_config2(edge=64, w=36, h=28, seed=17)
    z, y, x = shape
    cfg.voxels = np.ascontiguousarray(cfg.voxels[:z, :y, :x])
    _compare_samples(ctx, orc, cfg, samples=(0, 2))
    _plain_equals_wavefront(ctx, cfg)


@pytest.mark.parametrize("fill", [0, 1])
def test_empty_and_full_volumes(ctx, orc, fill):
    """Every ray misses (sky only), or every ray stops on the first voxel."""
    cfg = small_config1(edge=16, w=20, h=16, seed=18)
    cfg.voxels = np.full((13, 10, 17), fill, np.uint8)
    img = _compare_samples(ctx, orc, cfg, samples=(0, 1))
    assert np.isfinite(img).all()
    _plain_equals_wavefront(ctx, cfg)


def test_accumulation_matches_oracle_average(ctx, orc):
    cfg = small_config1(edge=48, w=40, h=32)
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        job.render(6)
        got = job.readback()
        osc, oenv = oracle_setup(orc, cfg, scene, env)
        want, _ = orc.render_average(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, 6, 32)
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
        assert job.samples() == 6
    finally:
        close_all(job, scene, env)


def test_kahan_accumulation_over_10k_samples(ctx):
    """10,000 samples of a frame with a sun and emissive voxels accumulate in
    FP32 with Kahan compensation to the float64 mean of the same per-sample
    radiance within 3 ulp, where a plain FP32 running sum drifts far more."""
    cfg = small_config2(edge=24, w=8, h=8)
    cfg.settings.max_samples = 1 << 20
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        n = 10000
        job.render(n)
        got = job.readback()[..., :3].astype(np.float64)
        exact = np.zeros((8, 8, 3))
        plain = np.zeros((8, 8, 3), np.float32)
        for k in range(n):
            rgb = job.samples_diag(k)[0][..., :3]
            exact += rgb
            plain += rgb
        exact /= n
        plain = plain.astype(np.float64) / n
        lit = exact > 1e-3
        err = np.abs(got - exact)[lit] / exact[lit]
        err_plain = np.abs(plain - exact)[lit] / exact[lit]
        assert lit.sum() > 100
        assert err.max() < 3 * 2.0 ** -23
        assert err_plain.max() > 10 * err.max()
    finally:
        close_all(job, scene, env)


def test_plain_and_persistent_kernels_agree(ctx):
    cfg = small_config2(edge=40, w=50, h=30)
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        ctx.set_kernel(1)
        job.render(5)
        a = job.readback().copy()
        job.reset()
        ctx.set_kernel(2)
        job.render(2)
        job.render(3)
        b = job.readback()
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    finally:
        ctx.set_kernel(2)
        close_all(job, scene, env)


def test_one_to_four_lanes_agree(ctx):
    """Two, three or four wavefront lanes on their own streams give the same
    bits as one."""
    cfg = small_config2(edge=40, w=96, h=80, seed=16)     # enough samples for four lanes
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        out = []
        for lanes in (1, 2, 3, 4):
            ctx.set_lanes(lanes)
            job.reset()
            job.render(3)
            out.append(job.readback().view(np.uint32).copy())
        for o in out[1:]:
            np.testing.assert_array_equal(out[0], o)
        with pytest.raises(L.VtError):
            ctx.set_lanes(5)
    finally:
        ctx.set_lanes(2)
        close_all(job, scene, env)


def test_graph_rounds_equal_direct_launches(ctx):
    """The wavefront rounds replayed from a captured graph give the same bits
    as the same rounds launched one by one."""
    cfg = small_config2(edge=32, w=48, h=40, seed=15)
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        out = []
        for graphs in (True, False, True):
            ctx.set_graphs(graphs)
            job.reset()
            job.render(5)
            out.append(job.readback().view(np.uint32).copy())
        np.testing.assert_array_equal(out[0], out[1])
        np.testing.assert_array_equal(out[0], out[2])
    finally:
        ctx.set_graphs(True)
        close_all(job, scene, env)


def test_batch_equals_alone(ctx):
    cfgs = [small_config1(edge=40, w=37, h=23, seed=5), small_config2(edge=32, w=64, h=48, seed=6),
            small_config1(edge=24, w=16, h=70, seed=7)]
    made = [gpu_setup(ctx, c) for c in cfgs]
    try:
        alone = []
        for _s, _e, j in made:
            j.render(4)
            alone.append(j.readback().copy())
            j.reset()
        ctx.render_batch([j for _s, _e, j in made], 2, path_slots=64)
        ctx.render_batch([j for _s, _e, j in made], 2, path_slots=96)
        for (_s, _e, j), want in zip(made, alone):
            np.testing.assert_array_equal(j.readback().view(np.uint32), want.view(np.uint32))
    finally:
        for m in made:
            close_all(m[2], m[0], m[1])


def test_server_results_equal_alone(ctx):
    cfgs = [small_config1(edge=40, w=30, h=20, seed=8), small_config2(edge=32, w=24, h=24, seed=9),
            small_config1(edge=32, w=40, h=10, seed=10)]
    spps = [5, 7, 3]
    made = [gpu_setup(ctx, c) for c in cfgs]
    # round_paths=1: no budget beyond the two passes each active request gets per round
    srv = Server(ctx, hbm_budget_bytes=1 << 30, max_active_jobs=2, passes_per_round=2, round_paths=1)
    try:
        alone = []
        for (_s, _e, j), spp in zip(made, spps):
            for _ in range(spp):
                j.render(1)
            alone.append(j.readback().copy())
        tickets = [srv.submit(s, e, c.camera, c.settings, c.width, c.height, spp)
                   for (s, e, _j), c, spp in zip(made, cfgs, spps)]
        for t, want, c in zip(tickets, alone, cfgs):
            assert srv.wait(t, 60.0) == L.VT_OK
            got, secs = srv.result(t, c.width, c.height)
            assert secs >= 0.0
            np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        st = srv.stats()
        assert st.completed == 3 and st.failed == 0
    finally:
        srv.close()
        for m in made:
            close_all(m[2], m[0], m[1])


def test_server_round_budget_goes_to_the_least_work_first(ctx):
    """A round's path budget: one pass each, then the rest to the request
    with the fewest paths left.  A 16x16x8 request and a 64x64x64 one share
    a budget of 64*64*8 + 16*16*8 paths: the small one finishes in the first
    round, the large one takes 8 passes a round, 8 rounds in all; both
    images equal the ones rendered alone."""
    cfgs = [small_config1(edge=32, w=16, h=16, seed=64), small_config1(edge=32, w=64, h=64, seed=65)]
    spps = [8, 64]
    made = [gpu_setup(ctx, c) for c in cfgs]
    srv = Server(ctx, max_active_jobs=4, passes_per_round=1, round_paths=64 * 64 * 8 + 16 * 16 * 8)
    try:
        alone = []
        for (_s, _e, j), spp in zip(made, spps):
            j.render(spp)
            alone.append(j.readback().copy())
        srv_paused = [srv.submit(s, e, c.camera, c.settings, c.width, c.height, spp)
                      for (s, e, _j), c, spp in zip(made, cfgs, spps)]
        for t, want, c in zip(srv_paused, alone, cfgs):
            assert srv.wait(t, 60.0) == L.VT_OK
            got, _ = srv.result(t, c.width, c.height)
            np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        # both requests may land in the first round or the second one in the
        # next: 8 rounds, or 9 when the small one ran alone first
        assert srv.stats().rounds in (8, 9)
    finally:
        srv.close()
        for m in made:
            close_all(m[2], m[0], m[1])


def test_server_quick_paths(ctx):
    """Requests whose remaining work fits quick_paths finish in one round,
    with the same images as rendered alone."""
    cfgs = [small_config1(edge=32, w=24, h=20, seed=61), small_config2(edge=32, w=20, h=16, seed=62)]
    spps = [9, 6]
    made = [gpu_setup(ctx, c) for c in cfgs]
    srv = Server(ctx, max_active_jobs=4, passes_per_round=2, quick_paths=1 << 20)
    try:
        alone = []
        for (_s, _e, j), spp in zip(made, spps):
            j.render(spp)
            alone.append(j.readback().copy())
        tickets = [srv.submit(s, e, c.camera, c.settings, c.width, c.height, spp)
                   for (s, e, _j), c, spp in zip(made, cfgs, spps)]
        for t, want, c in zip(tickets, alone, cfgs):
            assert srv.wait(t, 60.0) == L.VT_OK
            got, _ = srv.result(t, c.width, c.height)
            np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        assert srv.stats().rounds <= 2       # one round each at most, against 5 at two passes a round
    finally:
        srv.close()
        for m in made:
            close_all(m[2], m[0], m[1])


def test_server_round_paths_cap(ctx):
    """A request larger than the per-round cap advances one pass a round,
    with the same image as rendered alone."""
    cfg = small_config2(edge=32, w=32, h=32, seed=63)
    scene, env, job = gpu_setup(ctx, cfg)
    srv = Server(ctx, max_active_jobs=2, passes_per_round=4, round_paths_cap=1000)
    try:
        job.render(6)
        want = job.readback().copy()
        t = srv.submit(scene, env, cfg.camera, cfg.settings, 32, 32, 6)
        assert srv.wait(t, 60.0) == L.VT_OK
        got, _ = srv.result(t, 32, 32)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        assert srv.stats().rounds == 6       # 1024 pixels > 1000: one pass per round
    finally:
        srv.close()
        close_all(job, scene, env)


def test_server_admission_order(ctx):
    """One slot, a long request holding it, then a large and a small request
    queued behind it: arrival order finishes the large one first, least-work
    order the small one; the images do not depend on the order."""
    cfg = small_config1(edge=24, w=16, h=16, seed=11)
    scene, _env, job = gpu_setup(ctx, cfg)
    finished = {}
    images = {}
    try:
        for order in (L.VT_SERVE_ARRIVAL, L.VT_SERVE_LEAST_WORK):
            srv = Server(ctx, max_active_jobs=1, passes_per_round=4, order=order)
            try:
                t0 = time.perf_counter()
                sub = {}
                for name, res, spp in (("hold", 384, 256), ("large", 96, 64), ("small", 16, 4)):
                    sub[name] = (srv.submit(scene, None, cfg.camera, cfg.settings, res, res, spp),
                                 time.perf_counter() - t0, res)
                    if name == "hold":          # queue the others only once it holds the slot
                        for _ in range(2000):
                            if srv.poll(sub[name][0])[0] != L.VT_REQ_QUEUED:
                                break
                            time.sleep(0.001)
                        assert srv.poll(sub[name][0])[0] == L.VT_REQ_RUNNING
                done = {}
                for name, (t, at, res) in sub.items():
                    assert srv.wait(t, 120.0) == L.VT_OK
                    img, secs = srv.result(t, res, res)
                    done[name] = at + secs
                    images[(order, name)] = img.view(np.uint32).copy()
                finished[order] = done
            finally:
                srv.close()
        assert finished[L.VT_SERVE_ARRIVAL]["large"] < finished[L.VT_SERVE_ARRIVAL]["small"]
        assert finished[L.VT_SERVE_LEAST_WORK]["small"] < finished[L.VT_SERVE_LEAST_WORK]["large"]
        for name in ("hold", "large", "small"):
            np.testing.assert_array_equal(images[(L.VT_SERVE_ARRIVAL, name)], images[(L.VT_SERVE_LEAST_WORK, name)])
    finally:
        close_all(job, scene)


def _tri_soup(seed, n_small=3000, n_large=40, res=(96, 80, 64)):
    rng = np.random.default_rng(seed)
    ext = np.array(res, float)
    small = rng.uniform(0, 1, (n_small, 1, 3)) * ext
    small = small + rng.normal(0, 1.5, (n_small, 3, 3))
    large = rng.uniform(0, 1, (n_large, 3, 3)) * ext
    tris = np.concatenate([small, large]).reshape(-1, 3).astype(np.float32)
    # a few exact axis-aligned and degenerate triangles
    extra = np.array([[10, 10, 10], [30, 10, 10], [10, 30, 10], [5, 5, 5], [5, 5, 5], [9, 9, 9],
                      [20.5, 20.5, 20.0], [40.5, 20.5, 20.0], [20.5, 40.5, 20.0]], np.float32)
    v = np.concatenate([tris, extra])
    return v, np.arange(len(v), dtype=np.uint32)


@pytest.mark.parametrize("mode", [L.VT_VOXELIZE_THIN, L.VT_VOXELIZE_FAT,
                                  L.VT_VOXELIZE_THIN | L.VT_VOXELIZE_REFERENCE_BOUNDS,
                                  L.VT_VOXELIZE_FAT | L.VT_VOXELIZE_REFERENCE_BOUNDS])
def test_voxelize_bitexact_triangle_soup(ctx, orc, mode):
    v, idx = _tri_soup(3)
    for res in [(96, 80, 64), (97, 81, 66)]:            # the second one ends in partial bricks
        sc = Scene.voxelize(ctx, v, idx, res, mode=mode, placement=L.VT_MESH_VOXEL_SPACE)
        try:
            got = sc.voxels()
            want = orc.voxelize(v, idx, res, mode, placement=0)
            np.testing.assert_array_equal(got, want)
            assert want.sum() > 1000
            # the voxelizer sets the brick bits itself: they equal the layout's bricks of its voxels
            np.testing.assert_array_equal(sc.bricks(), bricks_from_voxels(want))
        finally:
            sc.close()


@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 2, 1), (1, 3, 2), (1, 1, 4), (4, 1, 1)])
def test_brick_shapes_trace_identically(ctx, shape):
    """Every brick shape: the bricks follow the layout of that shape, and a
    sample pass (first hits, per-sample radiance) and an accumulated frame are
    the same bits as with 4x4x4 bricks; edits keep the shape's bits."""
    cfg = small_config2(edge=37, w=40, h=32, seed=41)      # 37^3: partial bricks on every axis
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        base_rgba, base_hits, _ = job.samples_diag(0)
        job.render(3)
        base_img = job.readback().view(np.uint32).copy()
        scene.set_brick_shape(shape)
        assert scene.brick_shape() == tuple(shape)
        np.testing.assert_array_equal(scene.bricks(), bricks_from_voxels(cfg.voxels, shape))
        job.reset()
        rgba, hits, _ = job.samples_diag(0)
        assert np.array_equal(hits, base_hits)
        assert np.array_equal(rgba.view(np.uint32), base_rgba.view(np.uint32))
        job.render(3)
        assert np.array_equal(job.readback().view(np.uint32), base_img)
        scene.set_voxel(3, 4, 5, 0)
        scene.set_voxel(36, 36, 36, 1)
        want = cfg.voxels.copy()
        want[5, 4, 3] = 0
        want[36, 36, 36] = 1
        np.testing.assert_array_equal(scene.bricks(), bricks_from_voxels(want, shape))
        for bad in [(3, 3, 3), (3, 3, 0), (0, 2, 4), (5, 1, 0)]:
            with pytest.raises(L.VtError):
                scene.set_brick_shape(bad)
        assert scene.brick_shape() == tuple(shape)
    finally:
        close_all(job, scene, env)


def test_dense_scene_bricks_match_the_layout(ctx):
    rng = np.random.default_rng(5)
    for shape in [(64, 64, 64), (13, 30, 7), (5, 4, 9)]:
        g = (rng.random(shape) < 0.3).astype(np.uint8) * rng.integers(1, 3, size=shape, dtype=np.uint8)
        sc = Scene.dense(ctx, g, [S.lambert(0.5), S.lambert(0.2)])
        try:
            np.testing.assert_array_equal(sc.bricks(), bricks_from_voxels(g))
        finally:
            sc.close()


@pytest.mark.parametrize("mode", [L.VT_VOXELIZE_THIN, L.VT_VOXELIZE_FAT])
def test_voxelize_bitexact_icosphere(ctx, orc, mode):
    v, f = S.fbm_displaced_icosphere(level=5, seed=4)
    res = (128, 128, 128)
    sc = Scene.voxelize(ctx, v, f, res, mode=mode, placement=L.VT_MESH_FIT_UNIT_CUBE)
    try:
        got = sc.voxels()
        want = orc.voxelize(v, f, res, mode, placement=1)
        np.testing.assert_array_equal(got, want)
    finally:
        sc.close()


def test_voxelize_config5_full_size(ctx, orc):
    """The large-grid workload at its full size: the fBm-displaced icosphere
    of 1,310,720 triangles voxelized conservatively into 1024^3 equals the
    oracle bit for bit, and one sample per pixel of a 256^2 view of that
    volume (8 bounces) equals the oracle's per-sample radiance and first hits."""
    v, f = S.fbm_displaced_icosphere(level=8, seed=4)
    assert len(f) == 1310720
    res = (1024, 1024, 1024)
    sc = Scene.voxelize(ctx, v, f, res, mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE,
                        palette=[S.lambert(0.7)])
    job = None
    try:
        got = sc.voxels()
        want = orc.voxelize(v, f, res, L.VT_VOXELIZE_FAT, placement=1)
        assert np.array_equal(got, want)
        assert 4_000_000 < np.count_nonzero(want) < 6_000_000
        del want
        assert np.array_equal(sc.bricks(), bricks_from_voxels(got))
        cfg = S.config1(edge=8, width=256, height=256, spp=1)
        cfg.settings.max_bounces = 8
        job = Job(ctx, sc, None, cfg.camera, cfg.settings, 256, 256)
        rgba, hits, _ = job.samples_diag(0)
        osc = orc.Scene(got, [S.lambert(0.7)], None)
        wrgba, whits, _ = orc.render_samples(cfg.camera, cfg.settings, osc, orc.Env(), 256, 256, 0, 32)
        assert np.array_equal(hits, whits)
        assert np.array_equal(rgba.view(np.uint32), wrgba.view(np.uint32))
        assert ((hits[..., 3] >> 8) & 1).sum() > 10000      # the view sees the object
    finally:
        if job is not None:
            job.close()
        sc.close()


def test_emissive_discovery_in_voxel_order(ctx):
    """Discovery without pruning is exactly the emissive voxels in index
    order: a ragged volume of many discovery chunks, and one without lights."""
    rng = np.random.default_rng(31)
    g = rng.integers(0, 3, size=(61, 97, 150), dtype=np.uint8)          # 887,550 voxels
    g[rng.random(g.shape) < 0.03] = 3
    pal = [S.lambert(0.5), S.lambert(0.3), S.lambert(0.8, emission=(2.0, 1.0, 0.5))]
    sc = Scene.dense(ctx, g, pal, flags=L.VT_SCENE_AUTO_EMISSIVE)
    dark = Scene.dense(ctx, g, pal[:2] + [S.lambert(0.8)], flags=L.VT_SCENE_AUTO_EMISSIVE)
    try:
        np.testing.assert_array_equal(sc.emissive(), np.flatnonzero(g.ravel() == 3).astype(np.int32))
        assert dark.emissive().size == 0
    finally:
        sc.close()
        dark.close()


def test_emissive_pruning_matches_oracle(ctx, orc):
    cfg = small_config2(edge=48)
    sc = Scene.dense(ctx, cfg.voxels, cfg.palette, flags=L.VT_SCENE_AUTO_EMISSIVE | L.VT_SCENE_PRUNE_EMISSIVE)
    try:
        got = sc.emissive()
        cand = np.flatnonzero(cfg.voxels.ravel() == 17).astype(np.int32)
        want = orc.prune_emissive(cfg.voxels, cand)
        np.testing.assert_array_equal(got, want)
        assert 0 < len(got) < len(cand)
    finally:
        sc.close()


def test_pick_matches_oracle(ctx, orc):
    cfg = small_config1(edge=64, w=64, h=64)
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        osc, _ = oracle_setup(orc, cfg, scene, env)
        for x, y in [(32.5, 32.5), (10.0, 50.0), (0.5, 0.5), (60.2, 3.7)]:
            d, vox = job.pick(x, y)
            import ctypes as C
            od = C.c_float()
            ov = (C.c_int32 * 3)()
            orc.lib().orc_pick(C.byref(orc.camera(cfg.camera)), C.byref(orc.settings(cfg.settings)),
                               C.byref(osc.s), None, cfg.width, cfg.height, x, y, C.byref(od), ov)
            assert d == od.value and tuple(vox) == tuple(ov)
    finally:
        close_all(job, scene, env)


RMSE_CONFIGS = {
    "config1": lambda: small_config1(edge=64, w=64, h=64),
    "config2": lambda: small_config2(edge=48, w=48, h=40),
    "reference": lambda: reference_config(edge=40, w=40, h=32),
}


@pytest.mark.parametrize("name", list(RMSE_CONFIGS))
def test_converged_image_rmse_vs_fp64(ctx, orc, name):
    """Relative RMSE of the GPU's FP32 image against the oracle's FP64 build
    at equal sample counts, per configuration (printed for the record)."""
    cfg = RMSE_CONFIGS[name]()
    cfg.settings.max_samples = 1 << 20
    spp = 48
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        job.render(spp)
        got = job.readback()[..., :3].astype(np.float64)
        osc, oenv = oracle_setup(orc, cfg, scene, env)
        noise = ctx.noise_table() if cfg.settings.rng_mode == L.VT_RNG_NOISE_TABLE else None
        ref, _ = orc.render_average(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, spp, 64,
                                    noise=noise)
        ref = ref[..., :3].astype(np.float64)
        # with the reference's unguarded divisions a pixel that met a zero pdf
        # stays NaN (in either precision); the error is taken over the rest
        ok = np.isfinite(got).all(-1) & np.isfinite(ref).all(-1)
        rel_rmse = np.sqrt(np.mean((got[ok] - ref[ok]) ** 2)) / np.sqrt(np.mean(ref[ok] ** 2))
        print(f"relative RMSE vs FP64 oracle, {name}, {cfg.width}x{cfg.height} x {spp} spp: {rel_rmse:.3e} "
              f"({(~ok).sum()} non-finite pixels: {(~np.isfinite(got).all(-1)).sum()} FP32, "
              f"{(~np.isfinite(ref).all(-1)).sum()} FP64)")
        assert ok.mean() >= 0.95 if name == "reference" else ok.all()
        assert rel_rmse <= 1e-3, rel_rmse
    finally:
        close_all(job, scene, env)


def test_white_furnace_convex_box(ctx):
    """A convex object under a constant environment L = 1 with a Lambert
    albedo rho reflects exactly rho in expectation (NEE + MIS, no ground)."""
    g = np.zeros((32, 32, 32), np.uint8)
    g[8:24, 8:24, 8:24] = 1
    sc = Scene.dense(ctx, g, [S.lambert(0.6)])
    s = S.physical_settings(max_bounces=4)
    cam = S.orbit_camera(distance=1800.0, theta_deg=110.0, phi_deg=30.0)
    job = Job(ctx, sc, None, cam, s, 64, 64)
    try:
        job.render(256)
        img = job.readback()[..., :3]
        masks = [((job.samples_diag(k)[1][..., 3] >> 8) & 1).astype(bool) for k in range(8)]
        any_hit = np.logical_or.reduce(masks)
        all_hit = np.logical_and.reduce(masks)
        # pixels whose whole 3x3 neighbourhood always / never hit (silhouettes excluded)
        pad_any = np.pad(any_hit, 1, constant_values=True)
        pad_all = np.pad(all_hit, 1, constant_values=False)
        never = np.ones_like(any_hit)
        always = np.ones_like(any_hit)
        for dy in range(3):
            for dx in range(3):
                never &= ~pad_any[dy:dy + any_hit.shape[0], dx:dx + any_hit.shape[1]]
                always &= pad_all[dy:dy + any_hit.shape[0], dx:dx + any_hit.shape[1]]
        assert always.sum() > 200 and never.sum() > 200
        np.testing.assert_allclose(img[never], 1.0, rtol=0, atol=1e-6)
        assert abs(img[always].mean() - 0.6) < 0.01
    finally:
        close_all(job, sc)


ABLATIONS = ["base", "thinlens", "image_env", "metal", "emissive", "rr", "all"]


def _ablation_config(kind):
    from voxeltoy_gb300 import scenes as S2
    cfg = small_config1(edge=32, w=24, h=20, seed=12)
    rng = np.random.default_rng(3)
    if kind in ("thinlens", "all"):
        cfg.camera.lens_model = L.VT_LENS_THIN_LENS
        cfg.camera.lens_radius = 20.0
    if kind in ("image_env", "all"):
        cfg.env_rgb = S2.sky_sun_env(32, 16, peak=300.0)
    if kind in ("metal", "all"):
        cfg.palette = [S2.lambert(0.7), S2.metal(0.6, 0.2)]
        cfg.voxels = cfg.voxels * rng.integers(1, 3, size=cfg.voxels.shape, dtype=np.uint8)
    if kind in ("emissive", "all"):
        cfg.palette = list(cfg.palette) + [S2.lambert(0.5, emission=(5, 5, 5))]
        em = (rng.random(cfg.voxels.shape) < 0.05) & (cfg.voxels > 0)
        cfg.voxels = cfg.voxels.copy()
        cfg.voxels[em] = len(cfg.palette)
        cfg.scene_flags = L.VT_SCENE_AUTO_EMISSIVE | L.VT_SCENE_PRUNE_EMISSIVE
    if kind in ("rr", "all"):
        cfg.settings.rr_start_bounce = 1
    return cfg


@pytest.mark.parametrize("kind", ABLATIONS)
def test_samples_bitexact_ablation(ctx, orc, kind):
    cfg = _ablation_config(kind)
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        osc, oenv = oracle_setup(orc, cfg, scene, env)
        report = []
        for smp in (0, 1):
            g, gh, gc = job.samples_diag(smp)
            o, oh, oc = orc.render_samples(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, smp, 32)
            diff = ~same_bits(g, o)
            if diff.any() or not np.array_equal(gh, oh):
                px = np.argwhere(diff.any(axis=-1))
                rel = np.abs(g - o) / np.maximum(np.abs(o), 1e-30)
                y, x = px[0] if len(px) else (0, 0)
                report.append(f"sample {smp}: {len(px)} px differ, hits equal={np.array_equal(gh, oh)}, "
                              f"max rel {rel.max():.3e}, first ({x},{y}) gpu {g[y, x].tolist()} cpu {o[y, x].tolist()} "
                              f"counters gpu {gc[:7].tolist()} cpu {oc[:7].tolist()}")
        assert not report, "\n".join(report)
    finally:
        close_all(job, scene, env)


def _feature_configs():
    ref = reference_config(seed=6)                         # every quirk, noise-table RNG, thin lens, ground
    ref_img = reference_config(seed=7)
    ref_img.env_rgb = S.sky_sun_env(48, 24, peak=200.0)    # + image environment
    ortho = small_config1(edge=32, w=33, h=29, seed=8)     # orthographic, wireframe, selection
    ortho.camera.lens_model = L.VT_LENS_ORTHOGRAPHIC
    ortho.settings.wireframe_opacity = 0.6
    ortho.settings.wireframe_thickness = 0.05
    z, y, x = np.argwhere(ortho.voxels > 0)[len(np.argwhere(ortho.voxels > 0)) // 2]
    ortho.settings.selected_voxel[:] = [int(x), int(y), int(z)]
    ortho.settings.select_enabled = 1
    pin = small_config2(edge=40, w=31, h=17, seed=9)        # pinhole, RR, emissive NEE
    pin.camera.lens_model = L.VT_LENS_PINHOLE
    return {"reference": ref, "reference_image_env": ref_img, "ortho_wire_select": ortho, "pinhole": pin}


@pytest.mark.parametrize("name", ["reference", "reference_image_env", "ortho_wire_select", "pinhole"])
def test_wavefront_equals_plain_features(ctx, name):
    """Every camera model, quirk set and RNG through the wavefront kernels
    gives the same accumulation as the per-pixel kernel (itself bit-exact
    with the oracle per sample)."""
    cfg = _feature_configs()[name]
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        ctx.set_kernel(1)
        job.render(4)
        a = job.readback().copy()
        job.reset()
        ctx.set_kernel(2)
        job.render(4)
        np.testing.assert_array_equal(a.view(np.uint32), job.readback().view(np.uint32))
    finally:
        ctx.set_kernel(2)
        close_all(job, scene, env)


def test_batch_of_many_jobs_equals_alone(ctx):
    """More jobs than fit in the kernels' parameter block (the global job
    table), uneven sizes and different features, rendered alone and in one
    batch, and an empty batch."""
    cfgs = [small_config1(edge=16 + 4 * i, w=9 + 5 * i, h=7 + 3 * i, seed=20 + i) for i in range(7)]
    cfgs += list(_feature_configs().values())
    made = [gpu_setup(ctx, c) for c in cfgs]
    try:
        alone = []
        for _s, _e, j in made:
            j.render(3)
            alone.append(j.readback().copy())
            j.reset()
        assert len(made) > 8
        ctx.render_batch([j for _s, _e, j in made], 3)
        for (_s, _e, j), want in zip(made, alone):
            np.testing.assert_array_equal(j.readback().view(np.uint32), want.view(np.uint32))
        assert ctx.render_batch([], 3) == []
        before = [j.samples() for _s, _e, j in made]
        ctx.render_batch([j for _s, _e, j in made], 0)
        assert [j.samples() for _s, _e, j in made] == before
    finally:
        for s, e, j in made:
            close_all(j, s, e)


def test_full_size_config2(ctx, orc):
    """The benchmark's own frame: 256^3 fBm volume, 17 materials, 1024x512
    sky+sun environment, 1024^2 thin lens.  Per-sample radiance and first
    hits of two whole samples bit for bit against the oracle, and 8 spp
    accumulated identically by the wavefront in two lanes of 16M slots with
    CUDA graphs, in one lane of 1M slots without graphs, and by the plain
    kernel."""
    cfg = S.config2()
    _compare_samples(ctx, orc, cfg, samples=(0, 1))
    scene, env, job = gpu_setup(ctx, cfg)
    images = []
    try:
        for kernel, lanes, slots, graphs in ((2, 2, 1 << 25, 1), (2, 1, 1 << 20, 0), (1, 2, 0, 1)):
            ctx.set_kernel(kernel)
            ctx.set_lanes(lanes)
            ctx.set_graphs(graphs)
            if slots:
                ctx.set_tuning(slots, 0, 16)
            job.reset()
            job.render(8)
            images.append(job.readback().view(np.uint32).copy())
        for img in images[1:]:
            np.testing.assert_array_equal(img, images[0])
    finally:
        ctx.set_kernel(2)
        ctx.set_lanes(2)
        ctx.set_graphs(1)
        ctx.set_tuning(1 << 23, 0, 16)                 # the context defaults
        close_all(job, scene, env)



def test_counted_render_counters_agree_across_forms(ctx):
    """vt_diag_render_counted: the wavefront and plain forms count the same
    events of the same samples, and the wavefront's stream positions are one
    per path and round (at least one per path, at most one per bounce)."""
    cfg = small_config2(edge=40, w=48, h=40, seed=81)
    cfg.settings.max_samples = 1 << 20
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        wf = job.render_counted(6)
        job.reset()
        ctx.set_kernel(1)
        plain = job.render_counted(6)
        ctx.set_kernel(2)
        paths = 48 * 40 * 6
        assert wf[0] == plain[0] == paths
        np.testing.assert_array_equal(wf[:8], plain[:8])
        assert plain[8] == 0
        assert paths <= wf[8] <= paths * (cfg.settings.max_bounces + 1)
    finally:
        ctx.set_kernel(2)
        close_all(job, scene, env)


@pytest.mark.parametrize("steps", [4, 8, 16])
def test_pooled_trace_form_is_identical(ctx, steps):
    """The pooled DDA kernel (segment set-up for a warp's worth of records at
    once, lanes refilled from a shared-memory pool) gives the same images and
    event counters as the per-lane form: one job (parameter-block records),
    three jobs (parameter table) and eleven (global table)."""
    cfgs = [small_config2(edge=36, w=40, h=32, seed=90 + k) for k in range(11)]
    made = [gpu_setup(ctx, c) for c in cfgs]
    jobs = [m[2] for m in made]
    for c in cfgs:
        c.settings.max_samples = 1 << 20
    try:
        for group in (jobs[:1], jobs[:3], jobs):
            out = {}
            for form in (0, 1):
                ctx.set_trace_form(form)
                ctx.set_tuning(4096, -1, steps)
                for j in group:
                    j.reset()
                ctx.render_batch(group, 3)
                out[form] = [j.readback().view(np.uint32).copy() for j in group]
            for a, b in zip(out[0], out[1]):
                np.testing.assert_array_equal(a, b)
        ctx.set_trace_form(0)
        jobs[0].reset()
        c0 = jobs[0].render_counted(3)
        ctx.set_trace_form(1)
        jobs[0].reset()
        c1 = jobs[0].render_counted(3)
        np.testing.assert_array_equal(c0, c1)
    finally:
        ctx.set_trace_form(0)
        ctx.set_tuning(1 << 23, 0, 16)
        for m in made:
            close_all(m[2], m[0], m[1])


def test_volume_extent_limits_and_longest_rays(ctx, orc):
    """Volumes up to the documented extents (1,048,574 voxels along x and y,
    524,286 along z) are accepted, one more is refused with VT_EINVAL, and
    rays across the whole longest volume (a million DDA steps, distances in
    the millions) reach the same voxel as the oracle's."""
    pal = [S.lambert(0.5)]
    for shape in ((1, 1, 1048575), (1, 1048575, 1), (524287, 1, 1)):
        with pytest.raises(L.VtError) as e:
            Scene.dense(ctx, np.zeros(shape, np.uint8), pal)
        assert e.value.code == L.VT_EINVAL
    for shape in ((1, 1048574, 1), (524286, 1, 1)):
        Scene.dense(ctx, np.zeros(shape, np.uint8), pal).close()
    g = np.zeros((2, 2, 1048574), np.uint8)
    g[:, :, -1] = 1          # a wall at the far end
    g[1, 1, 700001] = 1      # and one voxel on the way
    cfg = small_config1(edge=8, w=8, h=8)
    cfg.voxels = g
    cfg.palette = pal
    scene, env, job = gpu_setup(ctx, cfg, env_rgb=None)
    try:
        inf = scene.info()
        lo, hi = np.array(inf.bounds_min, np.float32), np.array(inf.bounds_max, np.float32)
        c = (lo + hi) / 2
        q = (hi - lo) / 4
        x_near, x_far = lo[0] + 1e-3, lo[0] + np.float32(0.9) * (hi[0] - lo[0])
        o = np.array([[x_near, c[1] - q[1], c[2] - q[2]], [x_near, c[1] + q[1], c[2] + q[2]],
                      [x_far, c[1] + q[1], c[2] + q[2]], [x_near, c[1] + q[1], c[2] - q[2]]], np.float32)
        # long directions: dda.h raises a component below 1e-5 to 1e-5, so a
        # unit-length axis-aligned ray would leave the two-voxel rod after
        # 1e5 steps; with |d.x| = 1000 it drifts 1e-8 of a voxel per step
        d = np.array([[1000, 0, 0], [1000, 0, 0], [-1000, 0, 0], [1000, 1, 0]], np.float32)
        got = job.trace_rays(o, d)
        want = orc.trace_rays(orc.Scene(g, pal), o, d, 0)
        np.testing.assert_array_equal(got, want)
        hit = (got[:, 3] >> 8) & 1
        # the far wall 1,048,571 steps away; the voxel on the way, from either side
        assert hit[:3].all() and got[0, 0] == 1048573 and got[1, 0] == 700001 and got[2, 0] == 700001
    finally:
        close_all(job, scene, env)
