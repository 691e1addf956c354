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
  * hand-computed answers, on the oracle and on the CUDA traversal:
    axis-aligned rays, exact diagonals through voxel corners (all three
    axes step at once), grazing components, origins in an occupied voxel
    and outside the grid.
The GPU tests also compare the CUDA traversal with the double-precision
one directly.
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
        tmax[idx] += np.where(mask, tdel[idx], 0.0)
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


def voxel_point(res, ijk, frac=(0.5, 0.5, 0.5)):
    bmin, vs = world_bounds(res)
    return bmin + (np.array(ijk, float) + np.array(frac)) * vs


def unit(v):
    v = np.array(v, float)
    return v / np.linalg.norm(v)


def kat_cases():
    """(name, grid shape (x, y, z), occupied voxels, origin, direction,
    expected (hit, voxel, steps)), every answer worked out by hand."""
    cases = []
    res = (32, 32, 32)
    occ = [(20, 7, 9), (2, 7, 9), (3, 7, 25)]
    o = voxel_point(res, (10, 7, 9))
    cases += [("axis +x", res, occ, o, (1, 0, 0), (True, (20, 7, 9), 10)),
              ("axis -x", res, occ, o, (-1, 0, 0), (True, (2, 7, 9), 8)),
              # nothing along +y: leaves the grid after 32 - 7 steps
              ("axis +y", res, occ, o, (0, 1, 0), (False, (10, 32, 9), 25)),
              ("axis +z", res, occ, voxel_point(res, (3, 7, 0)), (0, 0, 1), (True, (3, 7, 25), 25))]
    # A ray along (1,1,1) through voxel corners crosses the three boundaries
    # at once and moves diagonally, so the face neighbours it passes at each
    # corner are never visited.
    occ = [(k, k - 1, k - 1) for k in range(1, 9)] + [(k - 1, k, k - 1) for k in range(1, 9)] + [(9, 9, 9)]
    cases.append(("diagonal", res, occ, voxel_point(res, (0, 0, 0), (0.25, 0.25, 0.25)), unit((1, 1, 1)),
                  (True, (9, 9, 9), 9)))
    # |d.y| <= 1e-5 becomes +1e-5 whatever its sign: from 5e-5 voxel below
    # the top face of row 12 such a ray climbs into row 13 within a few
    # voxels and hits the voxel there; d.y = -2e-5 keeps heading down.
    occ = [(30, 12, 4), (20, 13, 4)]
    o = voxel_point(res, (0, 12, 4), (0.5, 0.99995, 0.5))
    for dy in (-5e-6, 0.0, 5e-6):
        cases.append((f"grazing {dy:g}", res, occ, o, unit((1.0, dy, 0.0)), (True, (20, 13, 4), 21)))
    cases.append(("not grazing", res, occ, o, unit((1.0, -2e-5, 0.0)), (True, (30, 12, 4), 30)))
    res = (16, 16, 16)
    cases.append(("inside occupied", res, [(7, 6, 5)], voxel_point(res, (7, 6, 5)), (0.0, 0.6, 0.8),
                  (True, (7, 6, 5), 0)))
    return cases


def case_grid(res, occ):
    vox = np.zeros(res[::-1], np.uint8)
    for x, y, z in occ:
        vox[z, y, x] = 1
    return vox


@pytest.mark.parametrize("case", kat_cases(), ids=lambda c: c[0])
def test_hand_computed_rays(orc, case):
    _, res, occ, o, d, want = case
    vox = case_grid(res, occ)
    hit, p, steps = decode(orc.trace_rays(orc.Scene(vox, PAL), np.array([o], np.float32),
                                          np.array([d], np.float32)))
    assert (bool(hit[0]), tuple(int(c) for c in p[0]), int(steps[0])) == want
    # the exact traversal agrees
    ehit, ep, esteps, _ = traverse_exact(vox, np.array([o], np.float32), np.array([d], np.float32))
    if case[0] != "not grazing" and not case[0].startswith("grazing"):
        assert (bool(ehit[0]), tuple(int(c) for c in ep[0]), int(esteps[0])) == want


def test_origin_outside_the_grid(orc):
    res = (16, 16, 16)
    vox = case_grid(res, [(7, 6, 5)])
    hit, _, steps = decode(orc.trace_rays(orc.Scene(vox, PAL), np.array([voxel_point(res, (-3, 6, 5))], np.float32),
                                          np.array([(1.0, 0.0, 0.0)], np.float32)))
    assert not hit[0] and steps[0] == 0


def _gpu_trace(ctx, vox, o, d):
    from voxeltoy_gb300 import Job, Scene
    from voxeltoy_gb300 import scenes as S
    sc = Scene.dense(ctx, vox, [S.lambert(0.5)])
    job = None
    try:
        job = Job(ctx, sc, None, S.orbit_camera(), S.physical_settings(max_bounces=1), 8, 8)
        return decode(job.trace_rays(o, d))
    finally:
        if job is not None:
            job.close()
        sc.close()


@pytest.mark.gpu
def test_hand_computed_rays_gpu(ctx):
    """The same answers from the CUDA traversal, through the C ABI."""
    for name, res, occ, o, d, want in kat_cases():
        hit, p, steps = _gpu_trace(ctx, case_grid(res, occ), np.array([o], np.float32), np.array([d], np.float32))
        assert (bool(hit[0]), tuple(int(c) for c in p[0]), int(steps[0])) == want, name


@pytest.mark.gpu
@pytest.mark.parametrize("res", [(64, 64, 64), (48, 32, 40)])
def test_random_rays_match_exact_traversal_gpu(ctx, res):
    rng = np.random.default_rng(sum(res))
    vox = scene(res, 1)
    bmin, vs = world_bounds(res)
    d = rng.normal(size=(200000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d[(np.abs(d) > 1e-4).all(1)].astype(np.float32)
    o = (bmin + rng.random(d.shape) * np.array(res) * vs).astype(np.float32)
    hit, p, steps, gap = traverse_exact(vox, o, d)
    ghit, gp, gsteps = _gpu_trace(ctx, vox, o, d)
    same = (ghit == hit) & (gsteps == steps) & (~hit | (gp == p).all(1))
    assert (~same).sum() <= 5
    assert (gap[~same] < 1e-5).all()
