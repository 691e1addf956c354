"""Shared set-up of matched GPU / oracle inputs for the parity tests."""
from __future__ import annotations

import math

import numpy as np

from voxeltoy_gb300 import Env, Job, Scene
from voxeltoy_gb300 import _lib as L
from voxeltoy_gb300 import scenes as S


def small_config1(edge=64, w=48, h=40, seed=1):
    cfg = S.config1(edge=edge, width=w, height=h, spp=4, seed=seed)
    return cfg


def small_config2(edge=48, w=40, h=36, seed=2):
    cfg = S.config2(edge=edge, width=w, height=h, spp=4, seed=seed, env_size=(64, 32))
    return cfg


def reference_config(edge=40, w=40, h=32, seed=3):
    """All reference behaviours on: gamma before averaging, implicit ground,
    gradient-pdf mismatch, double reflectance, IOR 7.3, exponent = roughness,
    thin lens without jitter, x10 emissive light samples, noise-table RNG."""
    g = S.sphere_union(edge, 6, seed)
    rng = np.random.default_rng(seed)
    vox = g * rng.integers(1, 5, size=g.shape, dtype=np.uint8)
    pal = [S.lambert((0.8, 0.3, 0.3)), S.metal((0.9, 0.8, 0.5), 20.0), (L.VT_MATERIAL_PLASTIC, (0, 0, 0),
           (0.2, 0.5, 0.9), 8.0), S.lambert((0.6, 0.6, 0.6), emission=(2.0, 1.5, 1.0))]
    from voxeltoy_gb300 import default_settings
    s = default_settings()
    s.max_bounces = 3
    s.max_samples = 1 << 20
    s.rng_mode = L.VT_RNG_NOISE_TABLE
    cam = S.orbit_camera(distance=1800.0, theta_deg=115.0, phi_deg=30.0, lens=L.VT_LENS_THIN_LENS, aperture=15.0)
    return S.RenderConfig("reference", vox, pal, cam, s, w, h, 4,
                          scene_flags=L.VT_SCENE_AUTO_EMISSIVE | L.VT_SCENE_PRUNE_EMISSIVE)


def gpu_setup(ctx, cfg, env_rgb="cfg"):
    scene = Scene.dense(ctx, cfg.voxels, cfg.palette, flags=cfg.scene_flags)
    rgb = cfg.env_rgb if isinstance(env_rgb, str) else env_rgb
    env = Env(ctx, rgb) if rgb is not None else None
    job = Job(ctx, scene, env, cfg.camera, cfg.settings, cfg.width, cfg.height)
    return scene, env, job


def oracle_setup(orc, cfg, scene, env):
    """Oracle inputs: same volume and palette, the emissive list the GPU built
    (checked separately against the oracle's pruning), and the oracle's own
    environment build."""
    em = scene.emissive()
    osc = orc.Scene(cfg.voxels, cfg.palette, em if len(em) else None)
    oenv = orc.Env(cfg.env_rgb) if env is not None else orc.Env()
    return osc, oenv


def close_all(*objs):
    for o in objs:
        if o is not None:
            o.close()


def bricks_from_voxels(vox: np.ndarray, shape=(2, 2, 2)) -> np.ndarray:
    """The occupancy bit-bricks of a [z, y, x] volume as the library lays them
    out: one uint64 per brick of 2^sx x 2^sy x 2^sz voxels (shape = (sx, sy,
    sz)), bit (x & (2^sx-1)) | (y & (2^sy-1)) << sx | (z & (2^sz-1)) << (sx+sy),
    set for occupied voxels and for voxels outside the volume, on the brick
    grid padded by one all-set brick on every side."""
    sx, sy, sz = shape
    ex, ey, ez = 1 << sx, 1 << sy, 1 << sz
    rz, ry, rx = vox.shape
    bz, by, bx = -(-rz // ez), -(-ry // ey), -(-rx // ex)
    occ = np.ones(((bz + 2) * ez, (by + 2) * ey, (bx + 2) * ex), bool)
    occ[ez:ez + rz, ey:ey + ry, ex:ex + rx] = vox != 0
    blocks = occ.reshape(bz + 2, ez, by + 2, ey, bx + 2, ex).transpose(0, 2, 4, 1, 3, 5)   # [BZ,BY,BX,dz,dy,dx]
    bits = blocks.reshape(bz + 2, by + 2, bx + 2, 64).astype(np.uint64)
    weights = np.left_shift(np.uint64(1), np.arange(64, dtype=np.uint64))
    return (bits * weights).sum(-1, dtype=np.uint64)
