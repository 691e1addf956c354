"""C ABI behaviour on the GPU: budgets, validation, readback flags, the
reference's offset/table upload, the Renderer mirror, server admission,
cancellation and timeouts.  Failures are provoked on the host side (bad
arguments, a small budget, a cancelled request); nothing faults the GPU."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from helpers import close_all, gpu_setup, small_config1, small_config2
from voxeltoy_gb300 import Context, Env, Job, Renderer, Scene, Server
from voxeltoy_gb300 import _lib as L
from voxeltoy_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def test_budget_is_enforced_and_released():
    with Context(0, hbm_budget_bytes=32 << 20) as ctx:
        base = ctx.memory()
        with pytest.raises(L.VtError) as e:
            Scene.dense(ctx, np.zeros((320, 320, 320), np.uint8), [S.lambert(0.5)])
        assert e.value.code == L.VT_EBUDGET
        assert ctx.memory() == base
        sc = Scene.dense(ctx, np.ones((64, 64, 64), np.uint8), [S.lambert(0.5)])
        assert ctx.memory() > base
        sc.close()
        assert ctx.memory() == base


def test_input_validation(ctx):
    g = np.ones((8, 8, 8), np.uint8)
    with pytest.raises(L.VtError) as e:
        Scene.dense(ctx, g * 3, [S.lambert(0.5)])                       # entry 3 of a 1-entry palette
    assert e.value.code == L.VT_EINVAL
    with pytest.raises(L.VtError):
        Scene.dense(ctx, g, [(5, (0, 0, 0), (1, 1, 1), 0.0)])            # unknown material type
    with pytest.raises(L.VtError):
        Scene.dense(ctx, g, [S.lambert(0.5)], emissive=np.array([512], np.int32))
    bad = np.ones((4, 8, 3), np.float32)
    bad[1, 2, 0] = np.nan
    with pytest.raises(L.VtError):
        Env(ctx, bad)
    sc = Scene.dense(ctx, g, [S.lambert(0.5)])
    try:
        s = S.physical_settings(2)
        s.ground_material = 4
        with pytest.raises(L.VtError):
            Job(ctx, sc, None, S.orbit_camera(), s, 8, 8)
        s.ground_material = 0
        s.max_bounces = -1
        with pytest.raises(L.VtError):
            Job(ctx, sc, None, S.orbit_camera(), s, 8, 8)
    finally:
        sc.close()
    assert b"" != L.load().vt_last_error()


def test_offsets_upload_matches_palette_upload(ctx):
    """createVoxelDataTexture's layout: int32 record offsets and a float table."""
    cfg = small_config1(edge=32, w=24, h=24)
    # two records: Lambert at offset 0 (7 floats), metal at offset 7 (8 floats)
    table = np.array([0, 0, 0, 0, 0.7, 0.6, 0.5,
                      1, 0, 0, 0, 0.9, 0.8, 0.4, 0.3], np.float32)
    rng = np.random.default_rng(1)
    occ = cfg.voxels > 0
    which = rng.integers(0, 2, size=cfg.voxels.shape)
    offsets = np.where(occ, np.where(which == 0, 0, 7), -1).astype(np.int32)
    dense = np.where(occ, which + 1, 0).astype(np.uint8)
    palette = [S.lambert((0.7, 0.6, 0.5)), S.metal((0.9, 0.8, 0.4), 0.3)]
    a = Scene.from_offsets(ctx, offsets, table)
    b = Scene.dense(ctx, dense, palette)
    try:
        np.testing.assert_array_equal(a.voxels(), b.voxels())
        ja = Job(ctx, a, None, cfg.camera, cfg.settings, 24, 24)
        jb = Job(ctx, b, None, cfg.camera, cfg.settings, 24, 24)
        ja.render(3); jb.render(3)
        np.testing.assert_array_equal(ja.readback().view(np.uint32), jb.readback().view(np.uint32))
        ja.close(); jb.close()
    finally:
        a.close(); b.close()
    with pytest.raises(L.VtError):
        Scene.from_offsets(ctx, np.where(occ, 100, -1).astype(np.int32), table)   # offset beyond the table
    with pytest.raises(L.VtError):
        Scene.from_offsets(ctx, np.where(occ, 11, -1).astype(np.int32), table)    # record cut off by the end


def test_readback_flags(ctx, orc):
    cfg = small_config1(edge=32, w=20, h=12)
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        job.render(2)
        lin = job.readback()
        flip = job.readback(L.VT_READBACK_FLIP_Y)
        np.testing.assert_array_equal(flip, lin[::-1])
        tm = job.readback(L.VT_READBACK_TONEMAP)
        want = orc.builtins(2, np.ascontiguousarray(lin[..., :3] * np.float32(1.0)),
                            np.full(lin[..., :3].shape, np.float32(1.0) / np.float32(2.2), np.float32))
        np.testing.assert_array_equal(tm[..., :3], want)
        assert job.samples() == 2
        job.reset()
        assert job.samples() == 0
    finally:
        close_all(job, scene, env)


def test_max_samples_finishes(ctx):
    cfg = small_config1(edge=24, w=8, h=8)
    cfg.settings.max_samples = 5
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        assert job.render(3) == L.VT_SAMPLES_PENDING
        assert job.render(3) == L.VT_FINISHED_RENDERING
        assert job.samples() == 5
        assert job.render(1) == L.VT_FINISHED_RENDERING and job.samples() == 5
    finally:
        close_all(job, scene, env)


def test_renderer_mirror(tmp_path):
    r = Renderer()
    r.initialize()
    try:
        cfg = S.config1(edge=32, width=32, height=24)
        r.resize_frame(32, 24)
        r.load_volume(cfg.voxels, cfg.palette)
        cam = r.camera()
        for f, _t in L.Camera._fields_:
            v = getattr(cfg.camera, f)
            if hasattr(v, "__len__"):
                getattr(cam, f)[:] = list(v)
            else:
                setattr(cam, f, v)
        r.update_camera()
        r.render_settings().max_samples = 4
        r.render_settings().max_bounces = 3
        r.update_render_settings()
        n = 0
        while r.render() == 0:
            n += 1
        assert n == 3 and r.job.samples() == 4
        img = r.image()
        assert img.shape == (24, 32, 4) and np.isfinite(img).all()
        out = tmp_path / "frame.pfm"
        r.save_image(str(out))
        data = out.read_bytes()
        assert data.startswith(b"PF\n32 24\n-1.0\n") and len(data) == len(b"PF\n32 24\n-1.0\n") + 32 * 24 * 12
        d, vox = r.pick_focal_distance(16.0, 12.0)
        assert r.job.samples() == 0
        assert (d < 99999999.0) == (vox[0] >= 0)
        r.resize_frame(16, 16)
        assert r.image().shape == (16, 16, 4)
    finally:
        r.close()


def test_server_budget_cancel_and_timeout(ctx):
    cfg = small_config1(edge=32, w=64, h=64)
    scene = Scene.dense(ctx, cfg.voxels, cfg.palette)
    srv = Server(ctx, hbm_budget_bytes=1 << 20, max_active_jobs=1, passes_per_round=1)
    try:
        big = srv.submit(scene, None, cfg.camera, cfg.settings, 1024, 1024, 4)   # 48 MiB of buffers > 1 MiB
        assert srv.wait(big, 30.0) == L.VT_EBUDGET
        assert srv.poll(big)[0] == L.VT_REQ_FAILED
        long = srv.submit(scene, None, cfg.camera, cfg.settings, 64, 64, 1 << 20)
        queued = srv.submit(scene, None, cfg.camera, cfg.settings, 64, 64, 4)
        assert srv.wait(long, 0.05) == L.VT_ETIMEOUT
        srv.cancel(queued)
        srv.cancel(long)
        assert srv.wait(queued, 30.0) == L.VT_ECANCELLED
        assert srv.wait(long, 30.0) == L.VT_ECANCELLED
        ok = srv.submit(scene, None, cfg.camera, cfg.settings, 16, 16, 3)
        assert srv.wait(ok, 30.0) == L.VT_OK
        img, secs = srv.result(ok, 16, 16)
        assert np.isfinite(img).all() and secs > 0
        st = srv.stats()
        assert st.failed == 1 and st.cancelled == 2 and st.completed == 1
        assert st.rounds > 0 and st.round_us > 0
    finally:
        srv.close()
        scene.close()


def test_emissive_scene_renders_light(ctx):
    """A single emissive voxel lights its neighbourhood only through NEE."""
    g = np.zeros((16, 16, 16), np.uint8)
    g[:2, :, :] = 1
    g[5, 8, 8] = 2
    pal = [S.lambert(0.8), S.lambert(0.5, emission=(20, 20, 20))]
    sc = Scene.dense(ctx, g, pal, flags=L.VT_SCENE_AUTO_EMISSIVE | L.VT_SCENE_PRUNE_EMISSIVE)
    try:
        assert sc.emissive().tolist() == [8 + 16 * (8 + 16 * 5)]
        s = S.physical_settings(2, top=(0, 0, 0), bottom=(0, 0, 0))
        cam = S.orbit_camera(distance=1500, theta_deg=150, phi_deg=20)
        job = Job(ctx, sc, None, cam, s, 32, 32)
        job.render(32)
        img = job.readback()
        assert img[..., :3].max() > 1.0 and img[..., :3].min() == 0.0
        job.close()
    finally:
        sc.close()


def test_vox_scene_matches_decoded_volume(ctx):
    """vt_scene_create_from_vox == vt_scene_create of what vt_vox_decode returns."""
    from test_formats import vox_file
    from voxeltoy_gb300 import formats as F
    rng = np.random.default_rng(3)
    size = (20, 16, 12)
    pts = {tuple(rng.integers(0, s) for s in size) for _ in range(600)}
    vox = [(x, y, z, int(rng.choice([3, 17, 40, 254]))) for x, y, z in sorted(pts)]
    data = vox_file(size, vox)
    grid, pal = F.vox_decode(data)
    a = Scene.from_vox(ctx, data)
    b = Scene.dense(ctx, grid, pal)
    try:
        np.testing.assert_array_equal(a.voxels(), grid)
        cfg = small_config1(edge=8, w=16, h=16)
        ja = Job(ctx, a, None, cfg.camera, cfg.settings, 16, 16)
        jb = Job(ctx, b, None, cfg.camera, cfg.settings, 16, 16)
        ja.render(2); jb.render(2)
        np.testing.assert_array_equal(ja.readback().view(np.uint32), jb.readback().view(np.uint32))
        ja.close(); jb.close()
    finally:
        a.close(); b.close()


def test_obj_scene_matches_mesh_voxelization(ctx):
    """vt_scene_voxelize_obj == vt_scene_voxelize_mesh on the same triangles."""
    v, f = S.icosphere(2)
    v = np.ascontiguousarray(v, np.float32)
    text = "".join(f"v {x:.9g} {y:.9g} {z:.9g}\n" for x, y, z in v)
    text += "".join(f"f {a + 1} {b + 1} {c + 1}\n" for a, b, c in f)
    for mode in (L.VT_VOXELIZE_THIN, L.VT_VOXELIZE_FAT):
        a = Scene.voxelize_obj(ctx, text, (40, 40, 40), mode=mode)
        b = Scene.voxelize(ctx, v, f, (40, 40, 40), mode=mode, placement=L.VT_MESH_FIT_UNIT_CUBE)
        try:
            np.testing.assert_array_equal(a.voxels(), b.voxels())
            assert np.count_nonzero(a.voxels()) > 0
        finally:
            a.close(); b.close()


def test_voxelize_rejects_out_of_range_indices(ctx):
    """A triangle index at or past the vertex count fails the call with
    VT_EINVAL naming the largest such index (the check runs on the device,
    which skips those triangles); the context stays usable."""
    v, f = S.icosphere(2)
    v = np.ascontiguousarray(v, np.float32)
    bad = np.array(f, np.uint32)
    bad[5, 1] = len(v)
    bad[9, 2] = len(v) + 7
    sc = Scene.voxelize(ctx, v, f, (40, 40, 40), mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE)
    want = sc.voxels()
    sc.close()
    base = ctx.memory()   # the context's scratch is sized for this mesh now
    for placement in (L.VT_MESH_FIT_UNIT_CUBE, L.VT_MESH_VOXEL_SPACE):
        with pytest.raises(L.VtError) as e:
            Scene.voxelize(ctx, v * 10 + 20, bad, (40, 40, 40), mode=L.VT_VOXELIZE_FAT, placement=placement)
        assert e.value.code == L.VT_EINVAL and f"index {len(v) + 7} out of range" in str(e.value)
        assert ctx.memory() == base
    sc = Scene.voxelize(ctx, v, f, (40, 40, 40), mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE)
    try:
        assert np.count_nonzero(want) > 0
        np.testing.assert_array_equal(sc.voxels(), want)
    finally:
        sc.close()


def test_voxel_edits_match_a_rebuilt_scene(ctx):
    """set_voxel keeps grid, bricks and the emissive list equal to a scene
    built from the edited volume: same voxels, same emissive list, same image."""
    rng = np.random.default_rng(4)
    g = (rng.random((20, 24, 28)) < 0.3).astype(np.uint8) * rng.integers(1, 3, (20, 24, 28), dtype=np.uint8)
    pal = [S.lambert(0.6), S.lambert(0.4, emission=(3.0, 3.0, 3.0))]
    flags = L.VT_SCENE_AUTO_EMISSIVE | L.VT_SCENE_PRUNE_EMISSIVE
    a = Scene.dense(ctx, g, pal, flags=flags)
    edits = [(0, 0, 0, 2), (27, 23, 19, 1), (3, 4, 5, 0), (4, 4, 4, 2), (7, 8, 3, 0), (8, 8, 4, 2), (11, 12, 13, 0)]
    want = g.copy()
    for x, y, z, e in edits:
        a.set_voxel(x, y, z, e)
        want[z, y, x] = e
    b = Scene.dense(ctx, want, pal, flags=flags)
    try:
        np.testing.assert_array_equal(a.voxels(), want)
        assert sorted(a.emissive().tolist()) == sorted(b.emissive().tolist())
        cfg = small_config1(edge=8, w=24, h=20)
        ja = Job(ctx, a, None, cfg.camera, cfg.settings, 24, 20)
        jb = Job(ctx, b, None, cfg.camera, cfg.settings, 24, 20)
        ja.render(3); jb.render(3)
        np.testing.assert_array_equal(ja.readback().view(np.uint32), jb.readback().view(np.uint32))
        a.set_voxel(1, 1, 1, 2)                 # an edit after the job was built reaches it
        want[1, 1, 1] = 2
        c = Scene.dense(ctx, want, pal, flags=flags)
        jc = Job(ctx, c, None, cfg.camera, cfg.settings, 24, 20)
        ja.reset(); ja.render(2); jc.render(2)
        np.testing.assert_array_equal(ja.readback().view(np.uint32), jc.readback().view(np.uint32))
        for j in (ja, jb, jc):
            j.close()
        c.close()
        with pytest.raises(L.VtError):
            a.set_voxel(28, 0, 0, 1)
        with pytest.raises(L.VtError):
            a.set_voxel(0, 0, 0, 3)
    finally:
        a.close(); b.close()


def test_caller_emissive_list_drops_removed_voxels(ctx):
    g = np.ones((8, 8, 8), np.uint8)
    em = np.array([0, 9, 100], np.int32)
    sc = Scene.dense(ctx, g, [S.lambert(0.5, emission=(1, 1, 1))], emissive=em)
    try:
        sc.set_voxel(1, 1, 0, 0)                # linear index 9
        assert sorted(sc.emissive().tolist()) == [0, 100]
    finally:
        sc.close()


def test_select_add_remove_services(ctx):
    cfg = small_config1(edge=32, w=32, h=32)
    scene = Scene.dense(ctx, cfg.voxels, cfg.palette)
    job = Job(ctx, scene, None, cfg.camera, cfg.settings, 32, 32)
    try:
        x, y = 16.0, 16.0
        d0, v0 = job.pick(x, y)
        assert v0[0] >= 0
        sel, n = job.select_voxel(x, y)
        assert sel == v0 and sorted(abs(c) for c in n) in ([0.0, 0.0, 1.0], [0.0, 1.0, 1.0], [1.0, 1.0, 1.0])
        before = scene.voxels()
        # remove the voxel under the cursor: the pick now lands behind it
        job.render(2)
        assert job.remove_voxel(x, y) == v0 and job.samples() == 0
        vox = scene.voxels()
        assert vox[v0[2], v0[1], v0[0]] == 0
        assert np.count_nonzero(vox != before) == 1
        d1, v1 = job.pick(x, y)
        assert v1 != v0 and d1 >= d0
        # add on the new hit along its normal: the pick lands on the new voxel
        sel, n = job.select_voxel(x, y)
        new = job.add_voxel(x, y)
        assert new == tuple(s + int(c) for s, c in zip(sel, n))
        vox = scene.voxels()
        src = vox[sel[2], sel[1], sel[0]] if sel[1] >= 0 else cfg.settings.ground_material + 1
        assert vox[new[2], new[1], new[0]] == src
        assert job.pick(x, y)[1] == new
        # with screen-space motion the new voxel is offset along the camera right
        # axis's dominant components (several on ties, as the reference's step masks)
        sel, _ = job.select_voxel(x, y)
        moved = job.add_voxel(x, y, 5.0, 0.5)
        if moved[0] >= 0:
            off = [m - s for m, s in zip(moved, sel)]
            assert all(abs(o) <= 1 for o in off) and any(off)
        # nothing under the cursor: no edit
        vox = scene.voxels()
        assert job.remove_voxel(0.0, 0.0) == (-1, -1, -1) or job.pick(0.0, 0.0)[1][0] >= 0
    finally:
        job.close(); scene.close()


def test_zero_work_calls(ctx):
    """Zero passes, an empty batch and a job whose sample cap is reached leave
    the accumulation untouched; a job without samples reads back zeros."""
    cfg = small_config1(edge=16, w=8, h=6)
    cfg.settings.max_samples = 2
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        assert job.render(0) == L.VT_SAMPLES_PENDING and job.samples() == 0
        assert ctx.render_batch([], 3) == []
        assert ctx.render_batch([job], 0) == [L.VT_SAMPLES_PENDING] and job.samples() == 0
        np.testing.assert_array_equal(job.readback(), 0.0)
        assert job.render(5) == L.VT_FINISHED_RENDERING and job.samples() == 2
        done = job.readback().copy()
        assert job.render(3) == L.VT_FINISHED_RENDERING and job.samples() == 2
        np.testing.assert_array_equal(job.readback(), done)
    finally:
        close_all(job, scene, env)


def _offsets_scene_inputs():
    # records: Lambert at 0, metal at 7, an unused Lambert at 15, an emitting Lambert at 22
    table = np.array([0, 0, 0, 0, 0.8, 0.2, 0.2,
                      1, 0, 0, 0, 0.9, 0.9, 0.9, 30.0,
                      0, 0, 0, 0, 0.1, 0.6, 0.3,
                      0, 2.0, 2.0, 2.0, 0.5, 0.5, 0.5], np.float32)
    occ = S.sphere_union(24, 5, 41) > 0
    rng = np.random.default_rng(41)
    offsets = np.where(occ, rng.choice([0, 7, 22], size=occ.shape, p=[0.6, 0.35, 0.05]), -1).astype(np.int32)
    return offsets, table


def _image(ctx, scene, cfg, passes=2):
    job = Job(ctx, scene, None, cfg.camera, cfg.settings, cfg.width, cfg.height)
    try:
        job.render(passes)
        return job.readback().view(np.uint32).copy()
    finally:
        job.close()


def test_material_table_read_and_write(ctx):
    """Renderer::getMaterials / updateMaterialColor / updateMaterialValue:
    the caller's table comes back as given, and a scene whose table was
    written renders like a scene built from the written table."""
    cfg = small_config1(edge=24, w=24, h=20, seed=41)
    offsets, table = _offsets_scene_inputs()
    flags = L.VT_SCENE_AUTO_EMISSIVE
    sc = Scene.from_offsets(ctx, offsets, table, flags=flags)
    made = []
    try:
        np.testing.assert_array_equal(sc.material_table(), table)
        sc.write_material_table(4, [0.1, 0.9, 0.1])        # updateMaterialColor: albedo of record 0
        sc.write_material_table(14, 5.0)                    # updateMaterialValue: roughness of the metal
        sc.write_material_table(23, [0.0, 0.0, 0.0])        # the emitter goes dark
        sc.write_material_table(16, [3.0, 3.0, 3.0])        # emission of the unused record: table only
        want = table.copy()
        want[4:7] = [0.1, 0.9, 0.1]
        want[14] = 5.0
        want[23:26] = 0.0
        want[16:19] = 3.0
        np.testing.assert_array_equal(sc.material_table(), want)
        assert sc.emissive().size == 0
        ref = Scene.from_offsets(ctx, offsets, want, flags=flags)
        made.append(ref)
        np.testing.assert_array_equal(_image(ctx, sc, cfg), _image(ctx, ref, cfg))
        sc.write_material_table(23, [2.0, 2.0, 2.0])        # and lights up again
        lit = Scene.from_offsets(ctx, offsets, table, flags=flags)
        made.append(lit)
        assert lit.emissive().size > 0
        np.testing.assert_array_equal(sc.emissive(), lit.emissive())
        for off, n in ((0, 1), (5, 3), (15, 1), (29, 1), (-1, 1)):   # a type, across records, beyond the table
            with pytest.raises(L.VtError) as e:
                sc.write_material_table(off, np.zeros(n))
            assert e.value.code == L.VT_EINVAL
    finally:
        close_all(*made, sc)


def test_renderer_material_records(ctx):
    r = Renderer()
    r.ctx = ctx
    try:
        g = np.zeros((8, 8, 8), np.uint8)
        g[2:6, 2:6, 2:6] = 1
        g[0, 0, 0] = 2
        r.load_volume(g, [S.lambert((0.5, 0.4, 0.3)), S.metal((0.9, 0.8, 0.7), 12.0)], flags=0)
        recs = r.get_materials()
        assert [(o, t) for o, t, _ in recs] == [(0, L.VT_MATERIAL_LAMBERT), (7, L.VT_MATERIAL_METAL)]
        np.testing.assert_allclose(recs[1][2], [0, 0, 0, 0.9, 0.8, 0.7, 12.0], rtol=1e-6)
        r.update_material_color(4, (0.2, 0.2, 0.2))
        r.update_material_value(14, 40.0)
        recs = r.get_materials()
        np.testing.assert_allclose(recs[0][2][3:], [0.2, 0.2, 0.2], rtol=1e-6)
        assert recs[1][2][6] == 40.0
    finally:
        close_all(r.job, r.scene)


def test_contexts_on_two_threads(ctx):
    """Two contexts driven from two host threads at once (ctypes releases the
    GIL during library calls) give the images each gives alone."""
    import threading
    cfgs = [small_config1(edge=32, w=40, h=30, seed=51), small_config2(edge=32, w=36, h=28, seed=52)]

    def render(cfg, out, key):
        c = Context()
        try:
            sc, env, job = gpu_setup(c, cfg)
            try:
                for _ in range(3):
                    job.render(2)
                out[key] = job.readback().view(np.uint32).copy()
            finally:
                close_all(job, sc, env)
        finally:
            c.close()

    alone, both = {}, {}
    for i, cfg in enumerate(cfgs):
        render(cfg, alone, i)
    threads = [threading.Thread(target=render, args=(cfg, both, i)) for i, cfg in enumerate(cfgs)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i in range(len(cfgs)):
        np.testing.assert_array_equal(both[i], alone[i])


def test_server_teardown_returns_device_memory(ctx):
    """A server's own launch lane (wavefront buffers, sample buffer, graphs,
    lane streams) is freed with the server: create, serve and destroy three
    times and the device's free memory comes back."""
    import torch
    cfg = small_config1(edge=32, w=64, h=64, seed=71)
    scene, env, job = gpu_setup(ctx, cfg)
    try:
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for _ in range(3):
            srv = Server(ctx, max_active_jobs=2, passes_per_round=4, path_slots=1 << 20)
            t = srv.submit(scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height, 8)
            assert srv.wait(t, 60.0) == L.VT_OK
            srv.close()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] >= free0 - (64 << 20)
    finally:
        close_all(job, scene, env)



def test_snapshot_restore_resumes_bit_identically(ctx):
    """A job interrupted after 5 samples, snapshotted, destroyed and restored
    into a new job reaches 12 samples with the same bits as a job that was
    never interrupted (sums, compensations and the resolved image)."""
    cfg = small_config2(edge=32, w=40, h=28, seed=21)
    cfg.settings.max_samples = 1 << 20
    scene, env, whole = gpu_setup(ctx, cfg)
    part = Job(ctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    resumed = None
    try:
        whole.render(12)
        part.render(5)
        snap = part.snapshot()
        assert snap[2] == 5
        part.close()
        part = None
        resumed = Job(ctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
        resumed.restore(*snap)
        assert resumed.samples() == 5
        resumed.render(7)
        assert resumed.samples() == 12
        a, b = whole.snapshot(), resumed.snapshot()
        assert a[2] == b[2] == 12
        assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
        assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
        assert np.array_equal(whole.readback().view(np.uint32), resumed.readback().view(np.uint32))
        with pytest.raises(L.VtError) as e:
            resumed.restore(snap[0], snap[1], -1)
        assert e.value.code == L.VT_EINVAL
        with pytest.raises(L.VtError) as e:
            resumed.restore(snap[0][:10], snap[1][:10], 5)       # too small for the frame
        assert e.value.code == L.VT_EINVAL
        assert resumed.samples() == 12
    finally:
        close_all(*(j for j in (part, resumed) if j is not None), whole, scene, env)


def test_server_keeps_scenes_resident_and_evicts_lru(ctx):
    """vt_server_submit_dense: a volume is uploaded once per key, reused by
    later requests (no volume passed), evicted least recently used first
    when a new scene needs the budget, and its images equal renders of a
    caller-owned scene."""
    cfgs = [small_config1(edge=48, w=24, h=20, seed=71), small_config1(edge=40, w=24, h=20, seed=72),
            small_config1(edge=44, w=24, h=20, seed=73)]
    alone = []
    for c in cfgs:
        sc = Scene.dense(ctx, c.voxels, c.palette)
        j = Job(ctx, sc, None, c.camera, c.settings, c.width, c.height)
        j.render(3)
        alone.append(j.readback().copy())
        close_all(j, sc)
    job_bytes = 24 * 20 * 16 * 3
    scene_bytes = [c.voxels.size + 8 * ((c.voxels.shape[0] + 3) // 4 + 2) ** 3 + 16 + 4 for c in cfgs]
    # room for two of the scenes and a job, not for three
    budget = scene_bytes[0] + scene_bytes[2] + job_bytes + 4096
    srv = Server(ctx, hbm_budget_bytes=budget, max_active_jobs=1, passes_per_round=1)
    try:
        def run(key, cfg, with_volume):
            t = srv.submit_dense(key, cfg.voxels if with_volume else None, cfg.palette, cfg.camera, cfg.settings,
                                 cfg.width, cfg.height, 3)
            assert srv.wait(t, 60.0) == L.VT_OK
            return srv.result(t, cfg.width, cfg.height)[0]

        for img, want in [(run(10, cfgs[0], True), alone[0]), (run(10, cfgs[0], False), alone[0]),
                          (run(11, cfgs[1], True), alone[1])]:
            np.testing.assert_array_equal(img.view(np.uint32), want.view(np.uint32))
        st = srv.stats()
        assert (st.scene_uploads, st.scene_hits, st.scene_evictions, st.scenes_resident) == (2, 1, 0, 2)
        np.testing.assert_array_equal(run(10, cfgs[0], False).view(np.uint32), alone[0].view(np.uint32))
        # a third scene evicts the least recently used one (key 11), not key 10
        np.testing.assert_array_equal(run(12, cfgs[2], True).view(np.uint32), alone[2].view(np.uint32))
        st = srv.stats()
        assert (st.scene_uploads, st.scene_evictions, st.scenes_resident) == (3, 1, 2)
        with pytest.raises(L.VtError) as e:                       # key 11 is gone and no volume is given
            srv.submit_dense(11, None, cfgs[1].palette, cfgs[1].camera, cfgs[1].settings, 24, 20, 3)
        assert e.value.code == L.VT_EINVAL
        np.testing.assert_array_equal(run(10, cfgs[0], False).view(np.uint32), alone[0].view(np.uint32))
        assert srv.stats().bytes_in_use <= budget
    finally:
        srv.close()


def test_server_does_not_charge_caller_owned_scenes(ctx):
    """A scene the caller created is the caller's memory: a server whose
    budget is far below the scene's size still admits requests on it (only
    the job's buffers count)."""
    cfg = small_config1(edge=128, w=16, h=16, seed=74)
    sc = Scene.dense(ctx, cfg.voxels, cfg.palette)
    srv = Server(ctx, hbm_budget_bytes=64 << 10, max_active_jobs=2, passes_per_round=2)
    try:
        assert sc.info().device_bytes > 2 << 20
        t = srv.submit(sc, None, cfg.camera, cfg.settings, 16, 16, 2)
        assert srv.wait(t, 60.0) == L.VT_OK
        assert srv.stats().bytes_in_use == 0
    finally:
        srv.close()
        sc.close()


def test_released_memory_is_reused_and_trimmed():
    """A destroyed scene's device blocks serve the next scene of the same
    size without a new cudaMalloc; trim returns them; the budget counts live
    plus kept blocks; VT_DEVICE_NO_ALLOC_CACHE keeps nothing."""
    torch = pytest.importorskip("torch")
    g = np.zeros((256, 256, 256), np.uint8)
    g[:, :8, :] = 1
    with Context(0) as ctx:
        base = ctx.memory()
        Scene.dense(ctx, g, [S.lambert(0.5)]).close()
        assert ctx.memory() == base
        free1 = torch.cuda.mem_get_info(0)[0]
        sc = Scene.dense(ctx, g, [S.lambert(0.5)])
        free2 = torch.cuda.mem_get_info(0)[0]
        assert free1 - free2 < (4 << 20)   # the 16 MiB grid came from the kept blocks
        sc.close()
        assert ctx.trim() >= (16 << 20)
        assert torch.cuda.mem_get_info(0)[0] - free2 >= (16 << 20)
        assert ctx.trim() == 0
    with Context(0, hbm_budget_bytes=40 << 20) as ctx:
        Scene.dense(ctx, g, [S.lambert(0.5)]).close()                  # ~19 MiB kept
        g2 = np.zeros((320, 256, 256), np.uint8)
        sc = Scene.dense(ctx, g2, [S.lambert(0.5)])                  # ~22 MiB: fits after the kept blocks go
        sc.close()
    with Context(0, flags=L.VT_DEVICE_NO_ALLOC_CACHE) as ctx:
        Scene.dense(ctx, g, [S.lambert(0.5)]).close()
        assert ctx.trim() == 0
