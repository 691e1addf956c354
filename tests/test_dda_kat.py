"""Known answers for the oracle's voxel traversal (raymarch / traverse,
src/shaders/shared/dda.h:7-100), from an independent restatement.

The reference steps a float DDA in voxel space from the ray origin nudged by
sign(d) * 0.001 world units (dda.h:19), replaces direction components with
|d| <= 1e-5 by +1e-5 (:29), steps every axis whose boundary distance ties
for the minimum (:51-53) and stops on an occupied voxel, on leaving the grid
or after int(2 ceil(|res|)) steps (:98).  Checked here against:
  * Amanatides & Woo ("A Fast Voxel Traversal Algorithm for Ray Tracing",
    Eurographics 1987) in double precision on random rays, which must agree
    on the hit flag, the voxel and the step count except where the float
    traversal meets a near-tie (an origin within 1e-5 voxel of a voxel
    face, or two axis crossings within 1e-5 voxel of each other);
  * hand-computed answers: axis-aligned rays, exact diagonals through voxel
    corners (all three axes step at once), grazing components, origins in
    an occupied voxel and outside the grid.
"""
import numpy as np
import pytest

PAL = [(0, (0, 0, 0), (0.5, 0.5, 0.5), 0.0)]


def world_bounds(res):
    """createVoxelDataTexture's bounds (renderer.cpp:845-850): a cube of 1000
    units along the major axis, centred at 0, in float."""
    voxel = np.float32(1000.0) / np.float32(max(res))
    size = voxel * np.array(res, np.float32)
    return (-size * np.float32(0.5)).astype(np.float64), np.float64(voxel)


def step_cap(res):
    rx, ry, rz = (np.float32(r) for r in res)
    return int(np.float32(2.0) * np.ceil(np.sqrt(rx * rx + ry * ry + rz * rz)))


def traverse_exact(vox, o, d):
    """Amanatides-Woo in double from the nudged origin.  Returns the hit flag,
    the last voxel, the steps taken and, per ray, the nearest tie met on the
    way in voxels: the origin's distance to a voxel face, or the smallest gap
    between the two nearest axis crossings (in voxel-space t)."""
    rz, ry, rx = vox.shape
    res = np.array([rx, ry, rz])
    cap = step_cap((rx, ry, rz))
    bmin, vs = world_bounds((rx, ry, rz))
    d = d.astype(np.float64)
    o = o.astype(np.float64) + np.sign(d) * 0.001
    vo = (o - bmin) / vs
    p = np.floor(vo).astype(np.int64)
    step = np.sign(d).astype(np.int64)
    with np.errstate(divide="ignore"):
        tmax = np.where(d != 0, ((p + (step > 0)) - vo) / d, np.inf)
        tdel = np.where(d != 0, 1.0 / np.abs(d), np.inf)
    n = len(o)
    alive = np.ones(n, bool)
    hit = np.zeros(n, bool)
    steps = np.zeros(n, np.int64)
    gap = np.abs(vo - np.round(vo)).min(1)
    for s in range(cap + 1):
        alive &= (p >= 0).all(1) & (p < res).all(1)
        idx = np.nonzero(alive)[0]
        if idx.size == 0:
            break
        occ = vox[p[idx, 2], p[idx, 1], p[idx, 0]] != 0
        hit[idx[occ]] = True
        alive[idx[occ]] = False
        if s == cap:
            break
        idx = idx[~occ]
        tm = np.sort(tmax[idx], axis=1)
        gap[idx] = np.minimum(gap[idx], tm[:, 1] - tm[:, 0])
        mask = tmax[idx] == tm[:, :1]
        p[idx] += mask * step[idx]
        tmax[idx] += mask * tdel[idx]
        steps[idx] += 1
    return hit, p, steps, gap


def decode(out):
    return ((out[:, 3] >> 8) & 1).astype(bool), out[:, :3], out[:, 3] >> 10


def scene(res, seed):
    rng = np.random.default_rng(seed)
    rx, ry, rz = res
    vox = (rng.random((rz, ry, rx)) < 0.01).astype(np.uint8)
    z, y, x = np.meshgrid(np.arange(rz), np.arange(ry), np.arange(rx), indexing="ij")
    vox[((x - rx / 2) ** 2 + (y - ry / 2) ** 2 + (z - rz / 2) ** 2) < (min(res) / 4) ** 2] = 1
    return vox


@pytest.mark.parametrize("res", [(64, 64, 64), (48, 32, 40)])
def test_random_rays_match_exact_traversal(orc, res):
    rng = np.random.default_rng(sum(res))
    vox = scene(res, 1)
    bmin, vs = world_bounds(res)
    n = 200000
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d[(np.abs(d) > 1e-4).all(1)].astype(np.float32)
    o = (bmin + rng.random(d.shape) * np.array(res) * vs).astype(np.float32)
    hit, p, steps, gap = traverse_exact(vox, o, d)
    ohit, op, osteps = decode(orc.trace_rays(orc.Scene(vox, PAL), o, d))
    same = (ohit == hit) & (osteps == steps) & (~hit | (op == p).all(1))
    assert 0.2 < hit.mean() < 0.6
    assert (~same).sum() <= 5
    assert (gap[~same] < 1e-5).all()


def one_ray(orc, vox, o, d):
    hit, p, steps = decode(orc.trace_rays(orc.Scene(vox, PAL), np.array([o], np.float32), np.array([d], np.float32)))
    return bool(hit[0]), tuple(int(c) for c in p[0]), int(steps[0])


def voxel_point(res, ijk, frac=(0.5, 0.5, 0.5)):
    bmin, vs = world_bounds(res)
    return bmin + (np.array(ijk, float) + np.array(frac)) * vs


def test_axis_aligned_rays(orc):
    res = (32, 32, 32)
    vox = np.zeros(res[::-1], np.uint8)
    vox[9, 7, 20] = 1          # (x, y, z) = (20, 7, 9)
    vox[9, 7, 2] = 1
    vox[25, 7, 3] = 1
    o = voxel_point(res, (10, 7, 9))
    assert one_ray(orc, vox, o, (1, 0, 0)) == (True, (20, 7, 9), 10)
    assert one_ray(orc, vox, o, (-1, 0, 0)) == (True, (2, 7, 9), 8)
    # nothing along +y: leaves the grid after 32 - 7 steps
    assert one_ray(orc, vox, o, (0, 1, 0)) == (False, (10, 32, 9), 25)
    assert one_ray(orc, vox, voxel_point(res, (3, 7, 0)), (0, 0, 1)) == (True, (3, 7, 25), 25)


def test_exact_diagonal_steps_all_axes_together(orc):
    """A ray along (1,1,1) through voxel corners crosses the three boundaries
    at once and moves diagonally, so the face neighbours it passes at a
    corner are never visited."""
    res = (32, 32, 32)
    vox = np.zeros(res[::-1], np.uint8)
    for k in range(1, 9):
        vox[k - 1, k - 1, k] = 1     # (k, k-1, k-1): the +x neighbour of each diagonal voxel
        vox[k - 1, k, k - 1] = 1     # (k-1, k, k-1)
    vox[9, 9, 9] = 1
    d = np.full(3, 1.0 / np.sqrt(3.0))
    assert one_ray(orc, vox, voxel_point(res, (0, 0, 0), (0.25, 0.25, 0.25)), d) == (True, (9, 9, 9), 9)
    hit, p, steps, gap = traverse_exact(vox, voxel_point(res, (0, 0, 0), (0.25, 0.25, 0.25))[None],
                                        d[None].astype(np.float32))
    assert hit[0] and tuple(p[0]) == (9, 9, 9) and steps[0] == 9 and gap[0] == 0.0


def test_grazing_component_is_replaced_by_plus_1e_5(orc):
    """|d.y| <= 1e-5 becomes +1e-5 whatever its sign: from 5e-5 voxel below
    the top face of row 12, such a ray climbs into row 13 within a few voxels
    and hits the voxel there; a ray with d.y = -2e-5 keeps heading down and
    stays in row 12."""
    res = (32, 32, 32)
    vox = np.zeros(res[::-1], np.uint8)
    vox[4, 12, 30] = 1         # (30, 12, 4)
    vox[4, 13, 20] = 1         # (20, 13, 4)
    o = voxel_point(res, (0, 12, 4), (0.5, 0.99995, 0.5))
    for dy, want in ((-5e-6, (True, (20, 13, 4), 21)), (0.0, (True, (20, 13, 4), 21)),
                     (5e-6, (True, (20, 13, 4), 21)), (-2e-5, (True, (30, 12, 4), 30))):
        d = np.array([1.0, dy, 0.0])
        assert one_ray(orc, vox, o, d / np.linalg.norm(d)) == want, dy


def test_origin_in_an_occupied_voxel_and_outside(orc):
    res = (16, 16, 16)
    vox = np.zeros(res[::-1], np.uint8)
    vox[5, 6, 7] = 1
    assert one_ray(orc, vox, voxel_point(res, (7, 6, 5)), (0.0, 0.6, 0.8)) == (True, (7, 6, 5), 0)
    # outside the volume: no traversal at all
    hit, _, steps = one_ray(orc, vox, voxel_point(res, (-3, 6, 5)), (1.0, 0.0, 0.0))
    assert not hit and steps == 0
