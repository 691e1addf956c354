"""Known answers for the oracle's voxelizer (cpuVoxelizer.cpp:42-303,
voxelize.gs:55-251) from an independent separating-axis triangle/box test
(Akenine-Moller 2001, in double precision).

FAT (conservative) voxelization marks a voxel when the closed voxel box and
the triangle intersect, evaluated in float.  So, on any grid shape, FAT lies
between the separating-axis results for boxes of half-size 0.5 - 1e-4 and
0.5 + 1e-4: only voxels within float rounding of mere contact may go either
way.  Such voxels are rare for triangles in general position and common
with vertices on a coarse lattice (many voxels touch a triangle only at an
edge or a corner).  THIN (6-separating) is a subset of FAT.
The reference's own scan range (VT_VOXELIZE_REFERENCE_BOUNDS) clamps each
triangle's range in its swizzled frame against the unswizzled resolution
and skips voxels that only touch an integer bound; its effect is restated
here independently.
"""
import numpy as np
import pytest

from voxeltoy_gb300 import _lib as L

FAT, THIN, REF = L.VT_VOXELIZE_FAT, L.VT_VOXELIZE_THIN, L.VT_VOXELIZE_REFERENCE_BOUNDS
GRIDS = [(40, 40, 40), (48, 40, 32), (32, 40, 48), (40, 48, 32)]


def soup(res, seed, n=400, lattice=None):
    """Small triangles scattered over (and a little beyond) the grid plus a
    few that span it, in voxel units.  Zero-area triangles are left out:
    both voxelizers define them as covering nothing the other way round."""
    rng = np.random.default_rng(seed)
    ext = np.array(res, float)
    c = rng.uniform(-0.05, 1.05, (n, 1, 3)) * ext
    t = np.concatenate([c + rng.normal(0, 2.0, (n, 3, 3)), rng.uniform(-0.2, 1.2, (12, 3, 3)) * ext])
    if lattice:
        t = np.round(t / lattice) * lattice
    t = t.astype(np.float32)
    n64 = np.cross((t[:, 1] - t[:, 0]).astype(np.float64), (t[:, 2] - t[:, 1]).astype(np.float64))
    t = t[np.abs(n64).sum(1) > 0].reshape(-1, 3)
    return t, np.arange(len(t), dtype=np.uint32)


EPS = 1e-4


def check_between(orc, fat, v, i, res, keep=True):
    inner = orc.voxelize_sat(v, i, res, half=0.5 - EPS).astype(bool) & keep
    outer = orc.voxelize_sat(v, i, res, half=0.5 + EPS).astype(bool) & keep
    assert not (inner & ~fat).any()
    assert not (fat & ~outer).any()
    return orc.voxelize_sat(v, i, res).astype(bool) & keep


@pytest.mark.parametrize("res", GRIDS)
def test_fat_matches_separating_axis(orc, res):
    for seed in range(3):
        v, i = soup(res, seed)
        fat = orc.voxelize(v, i, res, FAT).astype(bool)
        sat = check_between(orc, fat, v, i, res)
        assert sat.sum() > 5000
        assert (fat != sat).sum() <= 2                 # general position: rounding only at contact
        thin = orc.voxelize(v, i, res, THIN).astype(bool)
        assert not (thin & ~fat).any()
        assert thin.sum() < 0.7 * fat.sum()


@pytest.mark.parametrize("res", [(24, 24, 24), (28, 20, 16)])
@pytest.mark.parametrize("lattice", [1.0, 0.5, 0.25])
def test_fat_on_lattice_vertices_between_shrunk_and_grown(orc, res, lattice):
    v, i = soup(res, 7, n=600, lattice=lattice)
    fat = orc.voxelize(v, i, res, FAT).astype(bool)
    sat = check_between(orc, fat, v, i, res)
    assert (fat != sat).sum() <= 0.01 * sat.sum()


def test_triangle_in_an_integer_plane(orc):
    """A triangle lying in the plane z = 10 touches the voxel layers 9 and 10;
    FAT marks both.  The reference's floor/ceil range is empty along z for it,
    so with VT_VOXELIZE_REFERENCE_BOUNDS it marks nothing."""
    res = (32, 24, 20)
    v = np.array([[4, 4, 10], [24, 4, 10], [4, 20, 10]], np.float32)
    i = np.arange(3, dtype=np.uint32)
    fat = orc.voxelize(v, i, res, FAT)
    np.testing.assert_array_equal(fat, orc.voxelize_sat(v, i, res))
    assert set(np.nonzero(fat.any(axis=(1, 2)))[0].tolist()) == {9, 10}
    assert fat[9].sum() == fat[10].sum() > 150
    assert orc.voxelize(v, i, res, FAT | REF).sum() == 0


def _dominant_perm(t):
    """The swizzle voxelize.gs:55-76 picks: 0 looks down x (frame yzx), 1 down
    y (zxy), 2 down z, from n = cross(v1 - v0, v2 - v1) in float."""
    a, b = t[1] - t[0], t[2] - t[1]
    n = np.array([a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]], np.float32)
    ax, ay, az = np.abs(n)
    if ax >= ay and ax >= az:
        return 0
    if ay >= ax and ay >= az:
        return 1
    return 2


@pytest.mark.parametrize("res", [(32, 24, 16), (16, 32, 24), (24, 16, 32)])
def test_reference_bounds_clamp_unswizzled(orc, res):
    """With the reference's bounds a voxel survives only where its coordinate
    along each swizzled axis c is below the grid's size along the unswizzled
    axis c (and, as before, inside the grid)."""
    rng = np.random.default_rng(11)
    rx, ry, rz = res
    z, y, x = np.meshgrid(np.arange(rz), np.arange(ry), np.arange(rx), indexing="ij")
    frame = {0: (y, z, x), 1: (z, x, y), 2: (x, y, z)}
    lost = 0
    for _ in range(60):
        t = (rng.uniform(0.1, 0.9, (1, 3)) * np.array(res) + rng.normal(0, 5.0, (3, 3))).astype(np.float32)
        i = np.arange(3, dtype=np.uint32)
        s = frame[_dominant_perm(t)]
        keep = (s[0] < rx) & (s[1] < ry) & (s[2] < rz)
        ref = orc.voxelize(t, i, res, FAT | REF).astype(bool)
        sat = check_between(orc, ref, t, i, res, keep)
        assert (ref != sat).sum() <= 1
        check_between(orc, orc.voxelize(t, i, res, FAT).astype(bool), t, i, res)
        lost += int((orc.voxelize_sat(t, i, res).astype(bool) & ~keep).sum())
    assert lost > 100


def test_reference_bounds_equal_on_cubic_grids(orc):
    res = (40, 40, 40)
    for seed in range(2):
        v, i = soup(res, seed)
        v = v + np.float32(0.37)     # off the integers, where only the FAT range differs
        for mode in (THIN, FAT):
            np.testing.assert_array_equal(orc.voxelize(v, i, res, mode), orc.voxelize(v, i, res, mode | REF))


@pytest.mark.gpu
@pytest.mark.parametrize("res", [(40, 40, 40), (48, 40, 32)])
def test_gpu_fat_matches_separating_axis(ctx, orc, res):
    """The CUDA voxelizer through the C ABI against the separating-axis test
    directly, including triangles in an integer plane."""
    from voxeltoy_gb300 import Scene
    v, i = soup(res, 5)
    plane = np.array([[4, 4, 10], [24, 4, 10], [4, 20, 10]], np.float32)
    v = np.concatenate([v, plane])
    i = np.arange(len(v), dtype=np.uint32)
    sc = Scene.voxelize(ctx, v, i, res, mode=FAT, placement=L.VT_MESH_VOXEL_SPACE)
    try:
        fat = sc.voxels().astype(bool)
    finally:
        sc.close()
    sat = check_between(orc, fat, v, i, res)
    assert (fat != sat).sum() <= 2
