"""ctypes binding of the CPU oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import build as _build

f3 = C.c_float * 3
i3 = C.c_int32 * 3


class OrcCamera(C.Structure):
    _fields_ = [("eye", f3), ("target", f3), ("fov_y", C.c_float), ("near_distance", C.c_float),
                ("far_distance", C.c_float), ("focal_distance", C.c_float), ("lens_radius", C.c_float),
                ("lens_model", C.c_int32)]


class OrcSettings(C.Structure):
    _fields_ = [("max_bounces", C.c_int32), ("max_samples", C.c_int32), ("rr_start_bounce", C.c_int32),
                ("gamma", C.c_float), ("exposure", C.c_float), ("nee_emission_scale", C.c_float),
                ("wireframe_opacity", C.c_float), ("wireframe_thickness", C.c_float),
                ("background_top", f3), ("background_bottom", f3), ("background_rotation", C.c_float),
                ("selected_voxel", i3), ("select_enabled", C.c_int32), ("ground_material", C.c_int32),
                ("quirks", C.c_uint32), ("rng_mode", C.c_int32), ("seed", C.c_uint32), ("integrator", C.c_int32)]


class OrcMaterial(C.Structure):
    _fields_ = [("type", C.c_int32), ("emission", f3), ("albedo", f3), ("roughness", C.c_float)]


class OrcScene(C.Structure):
    _fields_ = [("res", i3), ("grid", C.c_void_p), ("palette", C.POINTER(OrcMaterial)), ("n_palette", C.c_int32),
                ("emissive", C.c_void_p), ("n_emissive", C.c_int64)]


class OrcEnv(C.Structure):
    _fields_ = [("w", C.c_int32), ("h", C.c_int32), ("texels", C.c_void_p), ("cdf_u", C.c_void_p),
                ("cdf_v", C.c_void_p), ("integral", C.c_float), ("cdf_w", C.c_int32), ("cdf_h", C.c_int32)]


_LIB = None


def lib() -> C.CDLL:
    """The oracle library (VT_ORACLE_SANITIZED=1 selects the AddressSanitizer /
    UndefinedBehaviorSanitizer build, which needs libasan preloaded)."""
    global _LIB
    if _LIB is None:
        import os
        path = _build.build(sanitize=os.environ.get("VT_ORACLE_SANITIZED") == "1")
        L = C.CDLL(str(path))
        P = C.c_void_p
        sig = {
            "orc_camera_uniforms": ([C.POINTER(OrcCamera), C.c_int32, C.c_int32, P], C.c_int),
            "orc_camera_default": ([C.POINTER(OrcCamera)], None),
            "orc_camera_orbit": ([C.POINTER(OrcCamera), C.c_float, C.c_float], None),
            "orc_settings_default": ([C.POINTER(OrcSettings)], None),
            "orc_render_samples": ([C.POINTER(OrcCamera), C.POINTER(OrcSettings), C.POINTER(OrcScene),
                                    C.POINTER(OrcEnv), P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P,
                                    P], C.c_int),
            "orc_render_average": ([C.POINTER(OrcCamera), C.POINTER(OrcSettings), C.POINTER(OrcScene),
                                    C.POINTER(OrcEnv), P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_int32, P, P], C.c_int),
            "orc_trace_rays": ([C.POINTER(OrcScene), P, P, C.c_int64, C.c_uint32, P], C.c_int),
            "orc_pick": ([C.POINTER(OrcCamera), C.POINTER(OrcSettings), C.POINTER(OrcScene), P, C.c_int32, C.c_int32,
                          C.c_float, C.c_float, C.POINTER(C.c_float), P], C.c_int),
            "orc_build_env": ([P, C.c_int32, C.c_int32, C.c_int32, P, P, P, C.POINTER(C.c_float)], C.c_int),
            "orc_build_env_ex": ([P, C.c_int32, C.c_int32, C.c_int32, C.c_uint32, P, P, P, C.POINTER(C.c_float), P],
                                 C.c_int),
            "orc_cdf_size": ([C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)], None),
            "orc_cdf_from_function": ([P, C.c_int32, C.c_int32, C.c_int32, P, P, C.POINTER(C.c_float)], C.c_int),
            "orc_cdf_reference_float": ([P, C.c_int32, C.c_int32, P, P], C.c_int),
            "orc_binary_search": ([P, C.c_int32, C.c_float], C.c_int32),
            "orc_voxelize": ([P, C.c_int64, P, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                              C.c_int32, P], C.c_int),
            "orc_voxelize_sat": ([P, C.c_int64, P, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_double, P], C.c_int),
            "orc_prune_emissive": ([P, P, P, C.c_int64], C.c_int64),
            "orc_noise_table": ([P], C.c_int),
            "orc_philox": ([P, P, P], None),
            "orc_builtins": ([C.c_int32, P, P, P, C.c_int64], C.c_int),
            "orc_bsdf_sample": ([C.c_int32, P, C.c_float, C.c_uint32, P, P, C.c_int64, P], C.c_int),
            "orc_bsdf_eval": ([C.c_int32, P, C.c_float, C.c_uint32, P, P, C.c_int64, P], C.c_int),
            "orc_env_sample": ([C.POINTER(OrcEnv), C.c_float, P, C.c_int64, P], C.c_int),
            "orc_env_eval": ([C.POINTER(OrcEnv), C.c_float, P, C.c_int64, P], C.c_int),
            "orc_noise_walk": ([P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P], C.c_int),
            "orc_generate_rays": ([C.POINTER(OrcCamera), C.POINTER(OrcSettings), C.c_int32, C.c_int32, P, P,
                                   C.c_int64, P], C.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def camera(cam) -> OrcCamera:
    """Copy any structure with the camera fields (e.g. the product's vt_camera)."""
    o = OrcCamera()
    for name, _t in OrcCamera._fields_:
        v = getattr(cam, name)
        if hasattr(v, "__len__"):
            getattr(o, name)[:] = list(v)
        else:
            setattr(o, name, v)
    return o


def settings(s, integrator: int = 0) -> OrcSettings:
    """The oracle's copy of render settings `s`; `integrator` 0 path tracer,
    1 edit mode (a job attribute in the library, vt_job_set_integrator)."""
    o = OrcSettings()
    for name, _t in OrcSettings._fields_:
        if name == "integrator":
            o.integrator = integrator
            continue
        v = getattr(s, name)
        if hasattr(v, "__len__"):
            getattr(o, name)[:] = list(v)
        else:
            setattr(o, name, v)
    return o


# Cameras and settings built by the oracle alone, with the signatures of
# voxeltoy_gb300.scenes.orbit_camera / physical_settings, so that a
# configuration generated with make=<this module> never loads the library.
def orbit_camera(distance: float = 2000.0, theta_deg: float = 120.0, phi_deg: float = 45.0, fov_deg: float = 45.0,
                 lens: int = 0, aperture: float = 0.0, focus: float | None = None) -> OrcCamera:
    cam = OrcCamera()
    lib().orc_camera_default(C.byref(cam))
    cam.target[:] = [0.0, 0.0, 0.0]
    cam.eye[:] = [0.0, 0.0, -distance]
    lib().orc_camera_orbit(C.byref(cam), math.radians(theta_deg), math.radians(phi_deg))
    cam.fov_y = math.radians(fov_deg)
    cam.lens_model = lens
    cam.lens_radius = aperture
    cam.focal_distance = distance if focus is None else focus
    return cam


def physical_settings(max_bounces: int, rr_start: int = -1, seed: int = 0, top=(1.0, 1.0, 1.0),
                      bottom=(1.0, 1.0, 1.0)) -> OrcSettings:
    s = OrcSettings()
    lib().orc_settings_default(C.byref(s))
    s.max_bounces = max_bounces
    s.max_samples = 1 << 30
    s.rr_start_bounce = rr_start
    s.quirks = 0
    s.nee_emission_scale = 1.0
    s.background_top[:] = list(top)
    s.background_bottom[:] = list(bottom)
    s.seed = seed
    return s


def emissive_list(voxels: np.ndarray, palette, prune: bool = True) -> np.ndarray:
    """Linear indices of the voxels whose palette entry emits, in voxel order,
    then pruned of voxels with no empty 6-neighbour (import.cpp:133-203)."""
    hot = [i + 1 for i, m in enumerate(palette) if sum(m[1]) > 0]
    cand = np.flatnonzero(np.isin(np.asarray(voxels).ravel(), hot)).astype(np.int32)
    return prune_emissive(voxels, cand) if prune else cand


class Scene:
    """Keeps the numpy buffers alive for the C structure."""

    def __init__(self, voxels: np.ndarray, palette, emissive: np.ndarray | None = None):
        self.grid = np.ascontiguousarray(voxels, dtype=np.uint8)
        rz, ry, rx = self.grid.shape
        self.pal = (OrcMaterial * max(1, len(palette)))()
        for i, (t, e, a, r) in enumerate(palette):
            self.pal[i].type = int(t)
            self.pal[i].emission[:] = list(e)
            self.pal[i].albedo[:] = list(a)
            self.pal[i].roughness = float(r)
        self.em = np.ascontiguousarray(emissive if emissive is not None else np.zeros(1, np.int32), dtype=np.int32)
        n_em = 0 if emissive is None else len(emissive)
        self.s = OrcScene(i3(rx, ry, rz), C.c_void_p(self.grid.ctypes.data), self.pal, len(palette),
                          C.c_void_p(self.em.ctypes.data), n_em)


def cdf_size(w: int, h: int) -> tuple:
    """The reference's CDF image size for a w x h environment (image.cpp:314-317)."""
    cw, ch = C.c_int32(), C.c_int32()
    lib().orc_cdf_size(w, h, C.byref(cw), C.byref(ch))
    return cw.value, ch.value


class Env:
    """flags bit 0 (reference_size): CDFs and integral from the image shrunk to
    at most 512 texels on its long axis, texels full size."""

    def __init__(self, rgb: np.ndarray | None = None, texels=None, cdf_u=None, cdf_v=None, integral=None,
                 chunk: int = 32, flags: int = 0):
        if rgb is None:
            self.e = OrcEnv(0, 0, None, None, None, 0.0, 0, 0)
            return
        rgb = np.ascontiguousarray(rgb, dtype=np.float32)
        h, w = rgb.shape[:2]
        if texels is None:
            cw, ch = cdf_size(w, h) if flags & 1 else (w, h)
            texels = np.empty((h, w, 4), np.uint16)
            cdf_u = np.empty((ch, cw + 1), np.float32)
            cdf_v = np.empty(ch + 1, np.float32)
            iv = C.c_float()
            size = np.zeros(2, np.int32)
            lib().orc_build_env_ex(_p(rgb), w, h, chunk, flags, _p(texels), _p(cdf_u), _p(cdf_v), C.byref(iv),
                                   _p(size))
            assert tuple(size) == (cw, ch)
            integral = iv.value
        self.texels = np.ascontiguousarray(texels, dtype=np.uint16)
        self.cdf_u = np.ascontiguousarray(cdf_u, dtype=np.float32)
        self.cdf_v = np.ascontiguousarray(cdf_v, dtype=np.float32)
        self.integral = float(integral)
        self.e = OrcEnv(w, h, _p(self.texels), _p(self.cdf_u), _p(self.cdf_v), self.integral,
                        self.cdf_u.shape[1] - 1, self.cdf_u.shape[0])


def noise_table() -> np.ndarray:
    out = np.empty((1024, 1024, 4), np.float32)
    lib().orc_noise_table(_p(out))
    return out


def render_samples(cam, s, scene: Scene, env: Env, width: int, height: int, sample: int, precision: int = 32,
                   threads: int = 0, noise: np.ndarray | None = None, integrator: int = 0):
    rgba = np.empty((height, width, 4), np.float32)
    hits = np.empty((height, width, 4), np.int32)
    cnt = np.zeros(8, np.uint64)
    rc = lib().orc_render_samples(C.byref(camera(cam)), C.byref(settings(s, integrator)), C.byref(scene.s),
                                  C.byref(env.e),
                                  _p(noise), width, height, sample, precision, threads, _p(rgba), _p(hits), _p(cnt))
    assert rc == 0
    return rgba, hits, cnt


def render_average(cam, s, scene: Scene, env: Env, width: int, height: int, spp: int, precision: int = 32,
                   threads: int = 0, rows=(0, 0), noise: np.ndarray | None = None, integrator: int = 0):
    rgba = np.zeros((height, width, 4), np.float32)
    cnt = np.zeros(8, np.uint64)
    rc = lib().orc_render_average(C.byref(camera(cam)), C.byref(settings(s, integrator)), C.byref(scene.s),
                                  C.byref(env.e),
                                  _p(noise), width, height, spp, precision, threads, rows[0], rows[1], _p(rgba),
                                  _p(cnt))
    assert rc == 0
    return rgba, cnt


def trace_rays(scene: Scene, origins: np.ndarray, dirs: np.ndarray, quirks: int = 0) -> np.ndarray:
    o = np.ascontiguousarray(origins, dtype=np.float32)
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    out = np.empty((o.shape[0], 4), np.int32)
    lib().orc_trace_rays(C.byref(scene.s), _p(o), _p(d), o.shape[0], quirks, _p(out))
    return out


def camera_uniforms(cam, width: int, height: int) -> np.ndarray:
    out = np.empty(52, np.float32)
    assert lib().orc_camera_uniforms(C.byref(camera(cam)), width, height, _p(out)) == 0
    return out


def cdf_from_function(func: np.ndarray, chunk: int = 32):
    func = np.ascontiguousarray(func, dtype=np.float32)
    h, w = func.shape
    cu = np.empty((h, w + 1), np.float32)
    cv = np.empty(h + 1, np.float32)
    iv = C.c_float()
    lib().orc_cdf_from_function(_p(func), w, h, chunk, _p(cu), _p(cv), C.byref(iv))
    return cu, cv, iv.value


def cdf_reference_float(func: np.ndarray):
    func = np.ascontiguousarray(func, dtype=np.float32)
    h, w = func.shape
    cu = np.empty((h, w + 1), np.float32)
    cv = np.empty(h + 1, np.float32)
    lib().orc_cdf_reference_float(_p(func), w, h, _p(cu), _p(cv))
    return cu, cv


def binary_search(cdf, u: float) -> int:
    c = np.ascontiguousarray(cdf, dtype=np.float32)
    return lib().orc_binary_search(_p(c), c.size, u)


def voxelize(vertices, indices, res, mode: int, placement: int = 0, threads: int = 0) -> np.ndarray:
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    i = np.ascontiguousarray(indices, dtype=np.uint32)
    rx, ry, rz = res
    g = np.empty((rz, ry, rx), np.uint8)
    lib().orc_voxelize(_p(v), v.size // 3, _p(i), i.size // 3, rx, ry, rz, mode, placement, threads, _p(g))
    return g


def voxelize_sat(vertices_voxel_space, indices, res, half: float = 0.5) -> np.ndarray:
    v = np.ascontiguousarray(vertices_voxel_space, dtype=np.float32)
    i = np.ascontiguousarray(indices, dtype=np.uint32)
    rx, ry, rz = res
    g = np.empty((rz, ry, rx), np.uint8)
    lib().orc_voxelize_sat(_p(v), v.size // 3, _p(i), i.size // 3, rx, ry, rz, half, _p(g))
    return g


def prune_emissive(voxels: np.ndarray, emissive: np.ndarray) -> np.ndarray:
    g = np.ascontiguousarray(voxels, dtype=np.uint8)
    rz, ry, rx = g.shape
    res = np.array([rx, ry, rz], np.int32)
    lst = np.ascontiguousarray(emissive, dtype=np.int32).copy()
    n = lib().orc_prune_emissive(_p(g), _p(res), _p(lst), lst.size)
    return lst[:n]


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.empty(4, np.uint32)
    lib().orc_philox(_p(c), _p(k), _p(out))
    return out


def bsdf_sample(material, wo, u, quirks: int = 0):
    """material = (type, albedo[3], roughness); wo (n, 3) local, u (n, 2) ->
    wi (n, 3), f (n, 3), pdf (n,)."""
    t, a, r = material
    alb = np.ascontiguousarray(a, dtype=np.float32)
    w = np.ascontiguousarray(wo, dtype=np.float32)
    uu = np.ascontiguousarray(u, dtype=np.float32)
    out = np.empty((w.shape[0], 8), np.float32)
    assert lib().orc_bsdf_sample(int(t), _p(alb), float(r), quirks, _p(w), _p(uu), w.shape[0], _p(out)) == 0
    return out[:, :3], out[:, 3:6], out[:, 6]


def bsdf_eval(material, wo, wi, quirks: int = 0):
    t, a, r = material
    alb = np.ascontiguousarray(a, dtype=np.float32)
    w = np.ascontiguousarray(wo, dtype=np.float32)
    v = np.ascontiguousarray(wi, dtype=np.float32)
    out = np.empty((w.shape[0], 4), np.float32)
    assert lib().orc_bsdf_eval(int(t), _p(alb), float(r), quirks, _p(w), _p(v), w.shape[0], _p(out)) == 0
    return out[:, :3], out[:, 3]


def env_sample(env: Env, u, rotation: float = 0.0):
    """u (n, 2) -> dir (n, 3), radiance (n, 3), pdf (n,)."""
    uu = np.ascontiguousarray(u, dtype=np.float32)
    out = np.empty((uu.shape[0], 8), np.float32)
    assert lib().orc_env_sample(C.byref(env.e), rotation, _p(uu), uu.shape[0], _p(out)) == 0
    return out[:, :3], out[:, 3:6], out[:, 6]


def env_eval(env: Env, dirs, rotation: float = 0.0):
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    out = np.empty((d.shape[0], 4), np.float32)
    assert lib().orc_env_eval(C.byref(env.e), rotation, _p(d), d.shape[0], _p(out)) == 0
    return out[:, :3], out[:, 3]


def noise_walk(noise: np.ndarray, px: int, py: int, sample: int, n: int) -> np.ndarray:
    t = np.ascontiguousarray(noise, dtype=np.float32)
    out = np.empty((n, 4), np.float32)
    assert lib().orc_noise_walk(_p(t), px, py, sample, n, _p(out)) == 0
    return out


def generate_rays(cam, s, width: int, height: int, frag, u):
    """Camera rays for window positions frag (n, 2) and random blocks u (n, 4)
    -> origins (n, 3), directions (n, 3)."""
    f = np.ascontiguousarray(frag, dtype=np.float32)
    uu = np.ascontiguousarray(u, dtype=np.float32)
    out = np.empty((f.shape[0], 6), np.float32)
    assert lib().orc_generate_rays(C.byref(camera(cam)), C.byref(settings(s)), width, height, _p(f), _p(uu),
                                   f.shape[0], _p(out)) == 0
    return out[:, :3], out[:, 3:]


def builtins(fn: int, a, b=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a if b is None else np.ascontiguousarray(b, dtype=np.float32)
    out = np.empty_like(a)
    assert lib().orc_builtins(fn, _p(a), _p(b), _p(out), a.size) == 0
    return out
