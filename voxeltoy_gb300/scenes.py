"""Seeded synthetic inputs with the shapes of the benchmark configurations.

There is no public scene set for this path; these generators produce the
volumes, palettes, environment maps, cameras and meshes described by the
five benchmark configurations (all numpy, deterministic for a seed):

  config 1  64^3 union of 8 spheres + 4-voxel ground slab, one Lambert
            material (albedo 0.7), constant white environment, 256^2 pinhole.
  config 2  256^3 3-octave value-noise fBm thresholded at the 65th
            percentile (35% occupancy), 16-entry Lambert/Torrance-Sparrow
            palette + an emissive entry on 2% of occupied voxels, 1024^2
            thin lens, 1024x512 sky + sun environment, 8 bounces, RR after 3.
  config 3  64 sphere-union scenes, edges log-uniform in [32, 512].
  config 4  a Poisson request stream over config-1-style scenes.
  config 5  an icosphere displaced by fBm, voxelized conservatively.

Volumes are numpy arrays indexed [z, y, x]; voxel value 0 is empty and k
selects palette[k-1].  Sphere inclusion uses the voxel-centre distance rule
of src/renderer/content.cpp:46-52.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .renderer import default_camera, default_settings


# ---------------------------------------------------------------- volumes
def sphere_union(edge: int, n_spheres: int | None, seed: int, radius_range=(6.0, 16.0), slab: int = 4,
                 occupancy: float | None = None) -> np.ndarray:
    """Union of spheres (centres uniform in the grid, radii uniform in
    radius_range scaled by edge/64) plus a ground slab y in [0, slab*edge/64).
    With `occupancy`, spheres are added until that fraction is reached."""
    rng = np.random.default_rng(seed)
    g = np.zeros((edge, edge, edge), np.uint8)
    scale = edge / 64.0
    slab_h = max(1, int(round(slab * scale))) if slab else 0
    if slab_h:
        g[:, :slab_h, :] = 1
    coords = np.arange(edge, dtype=np.float32) + 0.5

    def stamp(c, r):
        lo = np.maximum(np.floor(c - r).astype(int), 0)
        hi = np.minimum(np.ceil(c + r).astype(int) + 1, edge)
        if np.any(hi <= lo):
            return
        dx = (coords[lo[0]:hi[0]] - c[0]) ** 2
        dy = (coords[lo[1]:hi[1]] - c[1]) ** 2
        dz = (coords[lo[2]:hi[2]] - c[2]) ** 2
        inside = (dz[:, None, None] + dy[None, :, None] + dx[None, None, :]) <= np.float32(r * r)
        sub = g[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
        sub[inside] = 1

    if occupancy is None:
        for _ in range(n_spheres):
            c = rng.uniform(0, edge, 3).astype(np.float32)
            r = np.float32(rng.uniform(*radius_range) * scale)
            stamp(c, r)
    else:
        total = float(edge) ** 3
        while np.count_nonzero(g) / total < occupancy:
            for _ in range(4):
                c = rng.uniform(0, edge, 3).astype(np.float32)
                r = np.float32(rng.uniform(*radius_range) * scale)
                stamp(c, r)
    return g


def value_noise_fbm(edge: int, octaves: int, seed: int, base_cells: int = 8, gain: float = 0.5) -> np.ndarray:
    """3-D fBm of value noise: random lattice values per octave, smoothstep
    trilinear interpolation, frequency doubling, amplitude * gain."""
    rng = np.random.default_rng(seed)
    out = np.zeros((edge, edge, edge), np.float32)
    amp = 1.0
    for o in range(octaves):
        cells = base_cells * (2 ** o)
        lattice = rng.random((cells + 1, cells + 1, cells + 1), dtype=np.float32)
        t = (np.arange(edge, dtype=np.float32) + 0.5) * (cells / edge)
        i0 = np.minimum(np.floor(t).astype(np.int64), cells - 1)
        f = t - i0
        s = f * f * (3.0 - 2.0 * f)
        # separable trilinear interpolation, x then y then z
        a = lattice[:, :, i0] * (1 - s)[None, None, :] + lattice[:, :, i0 + 1] * s[None, None, :]
        b = a[:, i0, :] * (1 - s)[None, :, None] + a[:, i0 + 1, :] * s[None, :, None]
        c = b[i0, :, :] * (1 - s)[:, None, None] + b[i0 + 1, :, :] * s[:, None, None]
        out += np.float32(amp) * c
        amp *= gain
    return out


def threshold_occupancy(field: np.ndarray, occupancy: float) -> np.ndarray:
    """Voxels above the (1-occupancy) quantile: exactly round(occupancy*N) voxels."""
    flat = field.ravel()
    k = int(round(occupancy * flat.size))
    idx = np.argpartition(flat, flat.size - k)[flat.size - k:]
    g = np.zeros(flat.size, np.uint8)
    g[idx] = 1
    return g.reshape(field.shape)


# -------------------------------------------------------------- palettes
def lambert(albedo, emission=(0.0, 0.0, 0.0)):
    a = albedo if np.ndim(albedo) else (albedo,) * 3
    return (L.VT_MATERIAL_LAMBERT, tuple(float(x) for x in emission), tuple(float(x) for x in a), 0.0)


def metal(f0, roughness, emission=(0.0, 0.0, 0.0)):
    a = f0 if np.ndim(f0) else (f0,) * 3
    return (L.VT_MATERIAL_METAL, tuple(float(x) for x in emission), tuple(float(x) for x in a), float(roughness))


def config2_palette(seed: int):
    rng = np.random.default_rng(seed + 1000)
    pal = [lambert(tuple(rng.uniform(0.2, 0.9, 3))) for _ in range(8)]
    pal += [metal(float(rng.uniform(0.04, 0.95)), float(rng.uniform(0.05, 0.5))) for _ in range(8)]
    pal.append(lambert((0.8, 0.8, 0.8), emission=(5.0, 5.0, 5.0)))   # emissive entry
    return pal


# ---------------------------------------------------------- environments
def sky_sun_env(width: int = 1024, height: int = 512, sun_elevation_deg: float = 40.0, sun_azimuth_deg: float = 30.0,
                sigma_deg: float = 1.0, peak: float = 1.0e4) -> np.ndarray:
    """Lat-long HDR map (row 0 = zenith): sky gradient 0.1 (horizon and below)
    to 1.0 (zenith) plus a Gaussian sun lobe of the given width and peak."""
    u = (np.arange(width, dtype=np.float64) + 0.5) / width
    v = (np.arange(height, dtype=np.float64) + 0.5) / height
    phi = u * 2 * math.pi - math.pi            # directionFromUVCoord, rotation 0
    theta = v * math.pi
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    d = np.stack([st * np.cos(phi)[None, :], np.broadcast_to(ct, (height, width)), st * np.sin(phi)[None, :]], -1)
    sky = 0.1 + 0.9 * np.clip(d[..., 1], 0.0, 1.0)
    el, az = math.radians(sun_elevation_deg), math.radians(sun_azimuth_deg)
    sun_dir = np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
    ang = np.arccos(np.clip(d @ sun_dir, -1.0, 1.0))
    lobe = peak * np.exp(-0.5 * (ang / math.radians(sigma_deg)) ** 2)
    rgb = sky[..., None] * np.array([0.6, 0.8, 1.0]) + lobe[..., None] * np.array([1.0, 0.95, 0.85])
    return rgb.astype(np.float32)


# ---------------------------------------------------------------- cameras
def orbit_camera(distance: float = 2000.0, theta_deg: float = 120.0, phi_deg: float = 45.0, fov_deg: float = 45.0,
                 lens: int = L.VT_LENS_PINHOLE, aperture: float = 0.0, focus: float | None = None) -> L.Camera:
    """Orbit camera around the volume centre.  The eye is placed at
    target - distance * sph(theta, phi) (CameraParameters::orbitAroundTarget),
    so theta > 90 degrees puts it above the volume."""
    cam = default_camera()
    cam.target[:] = [0.0, 0.0, 0.0]
    cam.eye[:] = [0.0, 0.0, -distance]
    L.call("vt_camera_orbit", C_byref(cam), math.radians(theta_deg), math.radians(phi_deg))
    cam.fov_y = math.radians(fov_deg)
    cam.lens_model = lens
    cam.lens_radius = aperture
    cam.focal_distance = distance if focus is None else focus
    return cam


def C_byref(x):
    import ctypes
    return ctypes.byref(x)


def physical_settings(max_bounces: int, rr_start: int = -1, seed: int = 0, top=(1.0, 1.0, 1.0),
                      bottom=(1.0, 1.0, 1.0)) -> L.RenderSettings:
    """Settings of the benchmark configurations: linear HDR accumulation, no
    implicit ground, per-material Fresnel F0 with exponent 2/r^2 - 2, thin-lens
    pixel jitter, emissive light samples without the x10 scale."""
    s = default_settings()
    s.max_bounces = max_bounces
    s.max_samples = 1 << 30
    s.rr_start_bounce = rr_start
    s.quirks = 0
    s.nee_emission_scale = 1.0
    s.background_top[:] = list(top)
    s.background_bottom[:] = list(bottom)
    s.seed = seed
    return s


# ----------------------------------------------------------------- configs
@dataclass
class RenderConfig:
    name: str
    voxels: np.ndarray
    palette: list
    camera: L.Camera
    settings: L.RenderSettings
    width: int
    height: int
    spp: int
    env_rgb: np.ndarray | None = None
    scene_flags: int = 0
    notes: dict = field(default_factory=dict)


def _maker(make):
    """Where cameras and settings come from: this module (the library's
    camera math), or any object with the same orbit_camera and
    physical_settings functions."""
    import sys
    return sys.modules[__name__] if make is None else make


def config1(edge: int = 64, width: int = 256, height: int = 256, spp: int = 16, seed: int = 1,
            make=None) -> RenderConfig:
    g = sphere_union(edge, 8, seed)
    mk = _maker(make)
    cam = mk.orbit_camera()
    s = mk.physical_settings(max_bounces=4, rr_start=-1, seed=seed)
    return RenderConfig("config1", g, [lambert(0.7)], cam, s, width, height, spp)


def config2(edge: int = 256, width: int = 1024, height: int = 1024, spp: int = 256, seed: int = 2,
            env_size=(1024, 512), make=None) -> RenderConfig:
    field_ = value_noise_fbm(edge, 3, seed)
    occ = threshold_occupancy(field_, 0.35)
    rng = np.random.default_rng(seed + 7)
    vox = occ * rng.integers(1, 17, size=occ.shape, dtype=np.uint8)
    emissive = (rng.random(occ.shape) < 0.02) & (occ > 0)
    vox[emissive] = 17
    mk = _maker(make)
    cam = mk.orbit_camera(lens=L.VT_LENS_THIN_LENS, aperture=0.02 * 1000.0)
    s = mk.physical_settings(max_bounces=8, rr_start=3, seed=seed)
    env = sky_sun_env(*env_size)
    return RenderConfig("config2", vox, config2_palette(seed), cam, s, width, height, spp, env_rgb=env,
                        scene_flags=L.VT_SCENE_AUTO_EMISSIVE | L.VT_SCENE_PRUNE_EMISSIVE)


def config3_scene(index: int) -> tuple[np.ndarray, int, int]:
    """Scene `index` of the batching configuration: (voxels, resolution, seed)."""
    seed = 100 + index
    rng = np.random.default_rng(seed)
    edge = int(round(math.exp(rng.uniform(math.log(32), math.log(512)))))
    occupancy = float(rng.uniform(0.10, 0.50))
    res = int(rng.choice([128, 256, 512, 1024]))
    return sphere_union(edge, None, seed, occupancy=occupancy), res, seed


# ------------------------------------------------------------------ meshes
def random_triangles(n: int, extent: float, seed: int, size: float = 3.0):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(size, extent - size, (n, 1, 3))
    tris = centres + rng.normal(0.0, size, (n, 3, 3))
    v = tris.reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.uint32)
    return v, idx


def icosphere(level: int):
    """Unit icosphere: 20 * 4^level triangles (level 8 -> 1,310,720)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid], 0)
        m = inv.reshape(3, -1).T + base   # midpoints of edges (01, 12, 20)
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                            np.stack([ab, bc, ca], 1)], 0)
    return v, f


def fbm_displaced_icosphere(level: int = 8, amplitude: float = 0.15, octaves: int = 4, seed: int = 4):
    """Icosphere whose vertices move radially by amplitude * fBm(p) (value
    noise on the unit sphere's bounding cube, in [-1, 1])."""
    v, f = icosphere(level)
    rng = np.random.default_rng(seed)
    disp = np.zeros(len(v))
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = 4 * 2 ** o
        lattice = rng.uniform(-1.0, 1.0, (cells + 1,) * 3)
        p = (v + 1.0) * 0.5 * cells
        i0 = np.minimum(np.floor(p).astype(np.int64), cells - 1)
        fr = p - i0
        s = fr * fr * (3 - 2 * fr)
        acc = np.zeros(len(v))
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    w = ((s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) *
                         (s[:, 2] if dz else 1 - s[:, 2]))
                    acc += w * lattice[i0[:, 2] + dz, i0[:, 1] + dy, i0[:, 0] + dx]
        disp += amp * acc
        total += amp
        amp *= 0.5
    disp /= total
    v = v * (1.0 + amplitude * disp)[:, None]
    return v.astype(np.float32), f.astype(np.uint32)
