"""A shading hit exactly on a voxel corner.

On the 1024^3 voxelization of the fBm-displaced icosphere (1.3M triangles),
rendered at 2048^2 with config-1 shading and 8 bounces, sample 216 of pixel
(1085, 1483) hits voxel (415, 971, 356) exactly on a corner.  All three axes
tie in the reference's normal (coordinates.h:74-75) and its tangent frame is
normalize(0), NaN, which poisons that pixel's average for good.  The
reference behaviour stays behind VT_QUIRK_UNGUARDED_SAMPLES; otherwise the
tie keeps one axis.  The oracle checks both; the GPU test checks the whole
2048^2 frame of that sample bit for bit against the oracle."""
import numpy as np
import pytest

from voxeltoy_gb300 import _lib as L
from voxeltoy_gb300 import scenes as S

PX, PY, SAMPLE = 1085, 1483, 216
RES = (1024, 1024, 1024)


@pytest.fixture(scope="module")
def mesh():
    v, f = S.fbm_displaced_icosphere(level=8)
    return np.ascontiguousarray(v, np.float32), np.ascontiguousarray(f, np.uint32)


@pytest.fixture(scope="module")
def oracle_grid(orc, mesh):
    v, f = mesh
    return orc.voxelize(v, f, RES, L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE)


def setup(quirks=0):
    cfg = S.config1(edge=8, width=2048, height=2048, spp=SAMPLE + 1)
    cfg.settings.max_bounces = 8
    cfg.settings.quirks = quirks
    return cfg


def test_oracle_corner_tie(orc, oracle_grid):
    sc = orc.Scene(oracle_grid, [S.lambert(0.7)], None)
    env = orc.Env()
    rows = (PY, PY + 1)
    guarded = setup()
    img, _ = orc.render_average(guarded.camera, guarded.settings, sc, env, 2048, 2048, SAMPLE + 1, rows=rows)
    assert np.isfinite(img[PY]).all()
    before, _ = orc.render_average(guarded.camera, guarded.settings, sc, env, 2048, 2048, SAMPLE, rows=rows)
    ref = setup(L.VT_QUIRK_UNGUARDED_SAMPLES)
    bad, _ = orc.render_average(ref.camera, ref.settings, sc, env, 2048, 2048, SAMPLE + 1, rows=rows)
    assert np.isnan(bad[PY, PX, :3]).all()
    # the other pixels of the row do not depend on the guard
    keep = np.ones(2048, bool)
    keep[PX] = False
    np.testing.assert_array_equal(bad[PY, keep].view(np.uint32), img[PY, keep].view(np.uint32))
    assert np.isfinite(before[PY, PX]).all()


@pytest.mark.gpu
def test_gpu_corner_tie_frame_bitexact(ctx, orc, mesh, oracle_grid):
    from helpers import close_all
    from voxeltoy_gb300 import Job, Scene
    v, f = mesh
    sc = Scene.voxelize(ctx, v, f, RES, mode=L.VT_VOXELIZE_FAT, placement=L.VT_MESH_FIT_UNIT_CUBE,
                        palette=[S.lambert(0.7)])
    job = None
    try:
        np.testing.assert_array_equal(sc.voxels() > 0, oracle_grid > 0)
        cfg = setup()
        job = Job(ctx, sc, None, cfg.camera, cfg.settings, 2048, 2048)
        rgba, hits, _ = job.samples_diag(SAMPLE)
        assert tuple(hits[PY, PX, :3]) == (415, 971, 356)
        assert np.isfinite(rgba[PY, PX]).all()
        osc = orc.Scene(oracle_grid, [S.lambert(0.7)], None)
        want, whits, _ = orc.render_samples(cfg.camera, cfg.settings, osc, orc.Env(), 2048, 2048, SAMPLE)
        np.testing.assert_array_equal(hits, whits)
        np.testing.assert_array_equal(rgba.view(np.uint32), want.view(np.uint32))
    finally:
        close_all(job, sc)
