"""Python mirror of voxelToy's Renderer interface over the C ABI.

``Renderer`` keeps the reference's verbs (src/renderer/renderer.h:23-221):
initialize, resize_frame, render (one progressive pass per call, returning
RR_SAMPLES_PENDING / RR_FINISHED_RENDERING), reset_render, camera(),
render_settings() + update_render_settings(), load_mesh, load_volume (the
createVoxelDataTexture upload), save_image and set_logger.  The lower-level
handles (Context, Scene, Env, Job, Server) map one to one onto vt.h.
All work runs in libvoxeltoy.so; nothing here computes pixels.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Sequence

import numpy as np

from . import _lib as L

RR_SAMPLES_PENDING = L.VT_SAMPLES_PENDING
RR_FINISHED_RENDERING = L.VT_FINISHED_RENDERING


def default_camera() -> L.Camera:
    cam = L.Camera()
    L.call("vt_camera_default", C.byref(cam))
    return cam


def default_settings() -> L.RenderSettings:
    s = L.RenderSettings()
    L.call("vt_settings_default", C.byref(s))
    return s


def camera_uniforms(cam: L.Camera, width: int, height: int) -> dict:
    u = L.CameraUniforms()
    L.call("vt_camera_compute_uniforms", C.byref(cam), width, height, C.byref(u))
    return {k: np.array(getattr(u, k), dtype=np.float32) for k in ("proj", "inv_proj", "inv_model_view", "viewport")}


class Context:
    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, flags: int = 0):
        L.load()
        opts = L.DeviceOpts(device, hbm_budget_bytes, flags)
        h = C.c_void_p()
        L.call("vt_create", C.byref(opts), C.byref(h))
        self.h = h
        self._log_cb = None

    def close(self):
        if self.h:
            L.call("vt_destroy", self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_logger(self, fn: Callable[[str], None] | None):
        self._log_cb = L.LOG_FN(lambda msg, _u: fn(msg.decode())) if fn else L.LOG_FN()
        L.call("vt_set_log_callback", self.h, self._log_cb, None)

    def memory(self) -> int:
        """Device bytes held for live objects (blocks kept for reuse excluded)."""
        v = C.c_uint64()
        L.call("vt_context_memory", self.h, C.byref(v))
        return v.value

    def trim(self) -> int:
        """Return the device memory kept for reuse; the bytes freed."""
        v = C.c_uint64()
        L.call("vt_context_trim", self.h, C.byref(v))
        return v.value

    def stream(self) -> int:
        st = C.c_void_p()
        L.call("vt_diag_stream", self.h, C.byref(st))
        return st.value or 0

    def set_tuning(self, path_slots: int = 0, trace_blocks_per_sm: int = -1, trace_steps: int = 0,
                   max_items: int = 0):
        """Wavefront launch parameters; 0 (or -1 for trace_blocks_per_sm) keeps a value."""
        L.call("vt_diag_set_tuning", self.h, path_slots, trace_blocks_per_sm, trace_steps, max_items)

    def set_trace_tuning(self, queue_chunk: int = 0, refill_min: int = -1):
        """DDA kernel parameters: queue records per warp atomic (32-1024, multiple
        of 32) and the early-refill threshold (0 = off); 0 / -1 keep a value."""
        L.call("vt_diag_set_trace_tuning", self.h, queue_chunk, refill_min)

    def set_trace_form(self, form: int):
        """DDA kernel form: 0 per-lane segment set-up, 1 pooled set-up (identical results)."""
        L.call("vt_diag_set_trace_form", self.h, form)

    def launch_count(self) -> int:
        n = C.c_uint64()
        L.call("vt_diag_launch_count", self.h, C.byref(n))
        return n.value

    def l2_read_bandwidth(self, nbytes: int = 32 << 20, reps: int = 1000) -> float:
        """GB/s of one launch of `reps` L1-bypassing read sweeps over an
        L2-resident buffer of `nbytes` bytes (vt_diag_l2_read_bandwidth)."""
        g = C.c_double()
        L.call("vt_diag_l2_read_bandwidth", self.h, nbytes, reps, C.byref(g))
        return g.value

    def set_kernel(self, kernel: int):
        L.call("vt_diag_set_kernel", self.h, kernel)

    def set_lanes(self, lanes: int):
        """Wavefront lanes side by side on their own streams (1-4; 2 is the default)."""
        L.call("vt_diag_set_lanes", self.h, lanes)

    def set_graphs(self, enabled: bool):
        """Replay wavefront rounds as a CUDA graph (default) or launch them one by one."""
        L.call("vt_diag_set_graphs", self.h, 1 if enabled else 0)

    def builtins(self, fn: int, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.float32)
        b = None if b is None else np.ascontiguousarray(b, dtype=np.float32)
        out = np.empty_like(a)
        L.call("vt_diag_builtins", self.h, fn, L.ptr(a), L.ptr(b), L.ptr(out), a.size)
        return out

    def cdf_from_function(self, func: np.ndarray):
        func = np.ascontiguousarray(func, dtype=np.float32)
        h, w = func.shape
        cu = np.empty((h, w + 1), np.float32)
        cv = np.empty(h + 1, np.float32)
        integral = C.c_float()
        L.call("vt_diag_cdf_from_function", self.h, L.ptr(func), w, h, L.ptr(cu), L.ptr(cv), C.byref(integral))
        return cu, cv, integral.value

    def noise_table(self) -> np.ndarray:
        out = np.empty((1024, 1024, 4), np.float32)
        L.call("vt_diag_get_noise_table", self.h, L.ptr(out), out.nbytes)
        return out

    def render_batch(self, jobs: Sequence["Job"], passes: int, path_slots: int = 0, kernel: int = 0,
                     blocks_per_sm: int = 0) -> list[int]:
        arr = (C.c_void_p * max(1, len(jobs)))(*[j.h.value for j in jobs])
        res = (C.c_int32 * max(1, len(jobs)))()
        opts = L.BatchOpts(path_slots, blocks_per_sm, 0, kernel)
        L.call("vt_render_batch", self.h, arr, len(jobs), passes, C.byref(opts), res)
        return list(res)[: len(jobs)]

    def render_batch_fixed(self, jobs: Sequence["Job"], passes: int, path_slots: int = 0) -> list[int]:
        """vt_render_batch_fixed: like render_batch with the wavefront kernels,
        with all working memory in the library's fixed device array (no
        allocation; calls must not overlap)."""
        arr = (C.c_void_p * max(1, len(jobs)))(*[j.h.value for j in jobs])
        res = (C.c_int32 * max(1, len(jobs)))()
        L.call("vt_render_batch_fixed", self.h, arr, len(jobs), passes, path_slots, res)
        return list(res)[: len(jobs)]


class Scene:
    def __init__(self, ctx: Context, handle: C.c_void_p):
        self.ctx = ctx
        self.h = handle

    @classmethod
    def dense(cls, ctx: Context, voxels: np.ndarray, palette, emissive: np.ndarray | None = None,
              flags: int = 0) -> "Scene":
        """voxels: uint8 array indexed [z, y, x] (0 empty, k = palette[k-1])."""
        v = np.ascontiguousarray(voxels, dtype=np.uint8)
        rz, ry, rx = v.shape
        pal = L.materials(palette)
        em = None if emissive is None else np.ascontiguousarray(emissive, dtype=np.int32)
        h = C.c_void_p()
        L.call("vt_scene_create", ctx.h, rx, ry, rz, L.ptr(v), pal, len(palette), L.ptr(em),
               0 if em is None else em.size, flags, C.byref(h))
        return cls(ctx, h)

    @classmethod
    def from_offsets(cls, ctx: Context, offsets: np.ndarray, table: np.ndarray, emissive: np.ndarray | None = None,
                     flags: int = 0) -> "Scene":
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        rz, ry, rx = off.shape
        t = np.ascontiguousarray(table, dtype=np.float32)
        em = None if emissive is None else np.ascontiguousarray(emissive, dtype=np.int32)
        h = C.c_void_p()
        L.call("vt_scene_create_from_offsets", ctx.h, rx, ry, rz, L.ptr(off), L.ptr(t), t.size, L.ptr(em),
               0 if em is None else em.size, flags, C.byref(h))
        return cls(ctx, h)

    @classmethod
    def voxelize(cls, ctx: Context, vertices: np.ndarray, indices: np.ndarray, resolution, mode: int = 1,
                 placement: int = L.VT_MESH_FIT_UNIT_CUBE, palette=None) -> "Scene":
        """Triangle mesh voxelized on the GPU (GPUVoxelizer::voxelizeMesh).  mode is
        VT_VOXELIZE_THIN or VT_VOXELIZE_FAT, optionally | VT_VOXELIZE_REFERENCE_BOUNDS
        for the reference's clamp of the swizzled scan range (drops voxels on
        non-cubic grids)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32)
        i = np.ascontiguousarray(indices, dtype=np.uint32)
        pal = palette or [(0, (0, 0, 0), (0.7, 0.7, 0.7), 0.0)]
        rx, ry, rz = resolution
        h = C.c_void_p()
        L.call("vt_scene_voxelize_mesh", ctx.h, L.ptr(v), v.size // 3, L.ptr(i), i.size // 3, rx, ry, rz, mode,
               placement, L.materials(pal), len(pal), C.byref(h))
        return cls(ctx, h)

    @classmethod
    def from_vox(cls, ctx: Context, data, flags: int = 0) -> "Scene":
        """MagicaVoxel .vox bytes or path (Renderer::loadVoxFile)."""
        from .formats import _bytes
        b = _bytes(data)
        h = C.c_void_p()
        L.call("vt_scene_create_from_vox", ctx.h, b, len(b), flags, C.byref(h))
        return cls(ctx, h)

    @classmethod
    def voxelize_obj(cls, ctx: Context, text, resolution=(64, 64, 64), mode: int = 0,
                     placement: int = L.VT_MESH_FIT_UNIT_CUBE, palette=None) -> "Scene":
        """Wavefront OBJ text or path, voxelized on the GPU (Renderer::loadMesh)."""
        from .formats import _bytes
        b = text.encode() if isinstance(text, str) and "\n" in text else _bytes(text)
        pal = palette or [(0, (0, 0, 0), (0.7, 0.7, 0.7), 0.0)]
        rx, ry, rz = resolution
        h = C.c_void_p()
        L.call("vt_scene_voxelize_obj", ctx.h, b, len(b), rx, ry, rz, mode, placement, L.materials(pal), len(pal),
               C.byref(h))
        return cls(ctx, h)

    def set_voxel(self, x: int, y: int, z: int, entry: int):
        """Edit one voxel: entry 0 empties it, k uses palette[k-1]."""
        L.call("vt_scene_set_voxel", self.h, x, y, z, entry)

    def info(self) -> L.SceneInfo:
        inf = L.SceneInfo()
        L.call("vt_scene_get_info", self.h, C.byref(inf))
        return inf

    def set_brick_shape(self, shape):
        """Log2 extents (sx, sy, sz) of the occupancy bricks, summing to 6."""
        L.call("vt_scene_set_brick_shape", self.h, *[int(v) for v in shape])

    def brick_shape(self) -> tuple:
        sh = (C.c_int32 * 3)()
        L.call("vt_scene_get_brick_shape", self.h, sh)
        return tuple(sh)

    def bricks(self) -> np.ndarray:
        """The occupancy bit-bricks on the padded brick grid ([bz+2, by+2, bx+2] uint64)."""
        n = C.c_int64()
        L.call("vt_diag_scene_bricks", self.h, None, 0, C.byref(n))
        out = np.empty(n.value, np.uint64)
        L.call("vt_diag_scene_bricks", self.h, L.ptr(out), out.nbytes, C.byref(n))
        rx, ry, rz = self.info().resolution
        sx, sy, sz = self.brick_shape()
        return out.reshape(((rz + (1 << sz) - 1) >> sz) + 2, ((ry + (1 << sy) - 1) >> sy) + 2,
                           ((rx + (1 << sx) - 1) >> sx) + 2)

    def voxels(self) -> np.ndarray:
        inf = self.info()
        rx, ry, rz = inf.resolution
        out = np.empty((rz, ry, rx), np.uint8)
        L.call("vt_scene_read_voxels", self.h, L.ptr(out), out.nbytes)
        return out

    def material_table(self) -> np.ndarray:
        """The materials as the reference's flat float table (type + data per record)."""
        n = C.c_int64()
        L.call("vt_scene_read_material_table", self.h, None, 0, C.byref(n))
        out = np.empty(max(1, n.value), np.float32)
        L.call("vt_scene_read_material_table", self.h, L.ptr(out), out.size, C.byref(n))
        return out[: n.value]

    def write_material_table(self, data_offset: int, values) -> None:
        v = np.ascontiguousarray(np.atleast_1d(values), dtype=np.float32)
        L.call("vt_scene_write_material_table", self.h, data_offset, L.ptr(v), v.size)

    def emissive(self) -> np.ndarray:
        n = C.c_int64()
        L.call("vt_scene_read_emissive", self.h, None, 0, C.byref(n))
        out = np.empty(max(1, n.value), np.int32)
        L.call("vt_scene_read_emissive", self.h, L.ptr(out), n.value, C.byref(n))
        return out[: n.value]

    def close(self):
        if self.h:
            L.call("vt_scene_destroy", self.h)
            self.h = None


class Env:
    def __init__(self, ctx: Context, rgb: np.ndarray, flags: int = 0):
        """flags: VT_ENV_CDF_REFERENCE_SIZE builds the CDFs from the image
        shrunk to at most 512 texels on its long axis, as the reference does."""
        img = np.ascontiguousarray(rgb, dtype=np.float32)
        self.h_px, self.w_px = img.shape[:2]
        h = C.c_void_p()
        L.call("vt_env_create_image_ex", ctx.h, L.ptr(img), self.w_px, self.h_px, flags, C.byref(h))
        self.h = h
        size = (C.c_int32 * 4)()
        L.call("vt_env_get_info", self.h, size)
        self.cdf_w, self.cdf_h = size[2], size[3]

    def cdf(self):
        cu = np.empty((self.cdf_h, self.cdf_w + 1), np.float32)
        cv = np.empty(self.cdf_h + 1, np.float32)
        integral = C.c_float()
        L.call("vt_env_read_cdf", self.h, L.ptr(cu), cu.nbytes, L.ptr(cv), cv.nbytes, C.byref(integral))
        return cu, cv, integral.value

    def texels(self) -> np.ndarray:
        out = np.empty((self.h_px, self.w_px, 4), np.uint16)
        L.call("vt_diag_env_texels", self.h, L.ptr(out), out.nbytes)
        return out

    def close(self):
        if self.h:
            L.call("vt_env_destroy", self.h)
            self.h = None


class Job:
    def __init__(self, ctx: Context, scene: Scene, env: Env | None, cam: L.Camera, settings: L.RenderSettings,
                 width: int, height: int):
        self.ctx, self.scene, self.env = ctx, scene, env
        self.width, self.height = width, height
        h = C.c_void_p()
        L.call("vt_job_create", ctx.h, scene.h, env.h if env else None, C.byref(cam), C.byref(settings), width,
               height, C.byref(h))
        self.h = h

    def render(self, passes: int = 1) -> int:
        r = C.c_int32()
        L.call("vt_job_render", self.h, passes, C.byref(r))
        return r.value

    def set_integrator(self, integrator: int):
        """VT_INTEGRATOR_PATH_TRACER or VT_INTEGRATOR_EDIT_MODE; restarts the accumulation."""
        L.call("vt_job_set_integrator", self.h, integrator)

    def render_counted(self, passes: int) -> np.ndarray:
        cnt = np.zeros(L.VT_DIAG_NUM_COUNTERS, np.uint64)
        r = C.c_int32()
        L.call("vt_diag_render_counted", self.h, passes, L.ptr(cnt), C.byref(r))
        return cnt

    def synchronize(self):
        L.call("vt_job_synchronize", self.h)

    def samples(self) -> int:
        n = C.c_int32()
        L.call("vt_job_sample_count", self.h, C.byref(n))
        return n.value

    def readback(self, flags: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 4), np.float32)
        L.call("vt_job_readback", self.h, L.ptr(out), out.nbytes, flags)
        return out

    def reset(self):
        L.call("vt_job_reset", self.h)

    def snapshot(self):
        """(sum, comp, samples): the accumulation state (vt_job_snapshot)."""
        sum_ = np.empty((self.height, self.width, 4), np.float32)
        comp = np.empty_like(sum_)
        n = C.c_int32()
        L.call("vt_job_snapshot", self.h, L.ptr(sum_), L.ptr(comp), sum_.nbytes, C.byref(n))
        return sum_, comp, n.value

    def restore(self, sum_: np.ndarray, comp: np.ndarray, samples: int):
        """Continue from a snapshot (vt_job_restore)."""
        s = np.ascontiguousarray(sum_, np.float32)
        c = np.ascontiguousarray(comp, np.float32)
        L.call("vt_job_restore", self.h, L.ptr(s), L.ptr(c), s.nbytes, samples)

    def set_camera(self, cam: L.Camera):
        L.call("vt_job_set_camera", self.h, C.byref(cam))

    def set_settings(self, s: L.RenderSettings):
        L.call("vt_job_set_settings", self.h, C.byref(s))

    def resize(self, width: int, height: int):
        L.call("vt_job_resize", self.h, width, height)
        self.width, self.height = width, height

    def pick(self, x: float, y: float):
        d = C.c_float()
        v = (C.c_int32 * 3)()
        L.call("vt_job_pick", self.h, x, y, C.byref(d), v)
        return d.value, tuple(v)

    def select_voxel(self, x: float, y: float):
        """(voxel, normal) under window point (x, y); voxel (-1, -1, -1) on a miss."""
        v = (C.c_int32 * 3)()
        n = (C.c_float * 3)()
        L.call("vt_job_select_voxel", self.h, x, y, v, n)
        return tuple(v), tuple(n)

    def add_voxel(self, x: float, y: float, dx: float = 0.0, dy: float = 0.0, restart: bool = True):
        v = (C.c_int32 * 3)()
        L.call("vt_job_add_voxel", self.h, x, y, dx, dy, 1 if restart else 0, v)
        return tuple(v)

    def remove_voxel(self, x: float, y: float, restart: bool = True):
        v = (C.c_int32 * 3)()
        L.call("vt_job_remove_voxel", self.h, x, y, 1 if restart else 0, v)
        return tuple(v)

    def samples_diag(self, sample: int):
        n = self.width * self.height
        rgba = np.empty((self.height, self.width, 4), np.float32)
        hits = np.empty((self.height, self.width, 4), np.int32)
        cnt = np.zeros(L.VT_DIAG_NUM_COUNTERS, np.uint64)
        L.call("vt_diag_samples", self.h, sample, L.ptr(rgba), L.ptr(hits), L.ptr(cnt))
        assert rgba.size == 4 * n
        return rgba, hits, cnt

    def trace_rays(self, origins: np.ndarray, dirs: np.ndarray) -> np.ndarray:
        o = np.ascontiguousarray(origins, dtype=np.float32)
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        out = np.empty((o.shape[0], 4), np.int32)
        L.call("vt_diag_trace_rays", self.h, L.ptr(o), L.ptr(d), o.shape[0], L.ptr(out))
        return out

    def close(self):
        if self.h:
            L.call("vt_job_destroy", self.h)
            self.h = None


class Server:
    def __init__(self, ctx: Context, hbm_budget_bytes: int = 0, max_active_jobs: int = 64,
                 passes_per_round: int = 4, path_slots: int = 0, order: int = L.VT_SERVE_ARRIVAL,
                 quick_paths: int = 0, round_paths_cap: int = 0, round_paths: int = 0):
        opts = L.ServerOpts(hbm_budget_bytes, max_active_jobs, passes_per_round, path_slots, order, quick_paths,
                            round_paths_cap, round_paths)
        h = C.c_void_p()
        L.call("vt_server_create", ctx.h, C.byref(opts), C.byref(h))
        self.h = h

    def submit(self, scene: Scene, env: Env | None, cam: L.Camera, settings: L.RenderSettings, width: int,
               height: int, spp: int) -> int:
        t = C.c_uint64()
        L.call("vt_server_submit", self.h, scene.h, env.h if env else None, C.byref(cam), C.byref(settings),
               width, height, spp, C.byref(t))
        return t.value

    def submit_dense(self, key: int, voxels: np.ndarray | None, palette, cam: L.Camera, settings: L.RenderSettings,
                     width: int, height: int, spp: int, env: Env | None = None, flags: int = 0,
                     shape=None) -> int:
        """vt_server_submit_dense: a request on a volume the server keeps
        resident under `key`; voxels may be None when the key is resident
        (then `shape` = (rz, ry, rx) is not needed either)."""
        t = C.c_uint64()
        if voxels is not None:
            v = np.ascontiguousarray(voxels, dtype=np.uint8)
            rz, ry, rx = v.shape
            pal = L.materials(palette)
            L.call("vt_server_submit_dense", self.h, key, rx, ry, rz, L.ptr(v), pal, len(palette), flags,
                   env.h if env else None, C.byref(cam), C.byref(settings), width, height, spp, C.byref(t))
        else:
            L.call("vt_server_submit_dense", self.h, key, 0, 0, 0, None, None, 0, flags,
                   env.h if env else None, C.byref(cam), C.byref(settings), width, height, spp, C.byref(t))
        return t.value

    def poll(self, ticket: int):
        st, n = C.c_int32(), C.c_int32()
        L.call("vt_server_poll", self.h, ticket, C.byref(st), C.byref(n))
        return st.value, n.value

    def wait(self, ticket: int, timeout_s: float = -1.0) -> int:
        return L.load().vt_server_wait(self.h, ticket, timeout_s)

    def result(self, ticket: int, width: int, height: int):
        out = np.empty((height, width, 4), np.float32)
        secs = C.c_double()
        L.call("vt_server_result", self.h, ticket, L.ptr(out), out.nbytes, C.byref(secs))
        return out, secs.value

    def cancel(self, ticket: int):
        L.call("vt_server_cancel", self.h, ticket)

    def stats(self) -> L.ServerStats:
        s = L.ServerStats()
        L.call("vt_server_get_stats", self.h, C.byref(s))
        return s

    def close(self):
        if self.h:
            L.call("vt_server_destroy", self.h)
            self.h = None


class Renderer:
    """voxelToy's Renderer verbs over one context, scene and job."""

    def __init__(self):
        self.ctx: Context | None = None
        self.scene: Scene | None = None
        self.env: Env | None = None
        self.job: Job | None = None
        self._camera = default_camera()
        self._settings = default_settings()
        self._integrator = L.VT_INTEGRATOR_PATH_TRACER
        self.width, self.height = 512, 512

    # Renderer::initialize (renderer.h:31)
    def initialize(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.ctx = Context(device, hbm_budget_bytes)

    def set_logger(self, fn):
        self.ctx.set_logger(fn)

    def camera(self) -> L.Camera:
        return self._camera

    def render_settings(self) -> L.RenderSettings:
        return self._settings

    # Renderer::createVoxelDataTexture (renderer.h:129-134)
    def load_volume(self, voxels: np.ndarray, palette, emissive=None, flags: int = L.VT_SCENE_PRUNE_EMISSIVE):
        self._replace_scene(Scene.dense(self.ctx, voxels, palette, emissive, flags))

    def load_volume_offsets(self, offsets: np.ndarray, table: np.ndarray, emissive=None, flags: int = 0):
        self._replace_scene(Scene.from_offsets(self.ctx, offsets, table, emissive, flags))

    # Renderer::loadMesh (renderer.h:60): voxelize into a res^3 grid
    def load_mesh(self, vertices: np.ndarray, indices: np.ndarray, resolution=(64, 64, 64), mode: int = 0):
        self._replace_scene(Scene.voxelize(self.ctx, vertices, indices, resolution, mode))

    # Renderer::loadMesh from an OBJ file (import.cpp:66-131)
    def load_mesh_file(self, path: str, resolution=(64, 64, 64), mode: int = 0):
        self._replace_scene(Scene.voxelize_obj(self.ctx, path, resolution, mode))

    # Renderer::loadVoxFile (renderer.h:62)
    def load_vox_file(self, path: str, flags: int = L.VT_SCENE_PRUNE_EMISSIVE):
        self._replace_scene(Scene.from_vox(self.ctx, path, flags))

    # Renderer::loadBackgroundImage (renderer.cpp:947-1055) from a PFM or Radiance HDR file
    def load_background_image(self, path: str):
        from .formats import image_decode
        self.set_background_image(image_decode(path))

    def set_background_image(self, rgb: np.ndarray | None):
        old = self.env
        self.env = Env(self.ctx, rgb) if rgb is not None else None
        if self.job:
            L.call("vt_job_set_scene", self.job.h, self.scene.h, self.env.h if self.env else None)
        if old:
            old.close()

    def _replace_scene(self, scene: Scene):
        old = self.scene
        self.scene = scene
        if self.job:
            L.call("vt_job_set_scene", self.job.h, scene.h, self.env.h if self.env else None)
        else:
            self.job = Job(self.ctx, scene, self.env, self._camera, self._settings, self.width, self.height)
            self.job.set_integrator(self._integrator)
        if old:
            old.close()

    # Renderer::getMaterials (renderer.h:120): (record offset, type, data) per
    # record of the flat material table, walked as the reference walks it
    def get_materials(self) -> list[tuple[int, int, np.ndarray]]:
        t = self.scene.material_table()
        out, at = [], 0
        while at < len(t) and t[at] in (0.0, 1.0, 2.0):
            n = 6 if t[at] == 0.0 else 7
            out.append((at, int(t[at]), t[at + 1: at + 1 + n].copy()))
            at += 1 + n
        return out

    # Renderer::updateMaterialColor / updateMaterialValue (renderer.h:121-122)
    def update_material_color(self, data_offset: int, color):
        self.scene.write_material_table(data_offset, np.asarray(color, np.float32)[:3])

    def update_material_value(self, data_offset: int, value: float):
        self.scene.write_material_table(data_offset, [value])

    # Renderer::resizeFrame (renderer.h:37-40)
    def resize_frame(self, width: int, height: int):
        self.width, self.height = width, height
        if self.job:
            self.job.resize(width, height)

    # Renderer::updateCamera + resetRender
    def update_camera(self):
        if self.job:
            self.job.set_camera(self._camera)

    # Renderer::updateRenderSettings (renderer.h:92)
    def update_render_settings(self):
        if self.job:
            self.job.set_settings(self._settings)

    # Renderer::onKeyPress(Qt::Key_Space) (renderer.cpp:678-683): path tracer <-> edit mode
    def toggle_integrator(self) -> int:
        self._integrator = 1 - self._integrator
        if self.job:
            self.job.set_integrator(self._integrator)
        return self._integrator

    # Renderer::resetRender (renderer.h:76)
    def reset_render(self):
        if self.job:
            self.job.reset()

    # Renderer::render (renderer.h:54): one progressive pass
    def render(self) -> int:
        if not self.job:
            return RR_FINISHED_RENDERING
        return self.job.render(1)

    def image(self, flags: int = 0) -> np.ndarray:
        return self.job.readback(flags)

    # Renderer::saveImage (renderer.h:72): float RGB written as a PFM file
    def save_image(self, path: str):
        """The accumulated image as a Radiance .hdr file (extension .hdr) or a PFM."""
        from .formats import encode_hdr, encode_pfm
        img = self.job.readback()                        # rows bottom first, as PFM stores them
        with open(path, "wb") as f:
            f.write(encode_hdr(img) if str(path).lower().endswith(".hdr") else encode_pfm(img))

    # Renderer::requestAction (renderer.h:106, actions.cpp:5-52): x, y and dx, dy
    # are normalised window coordinates with the origin at the top left, as
    # the reference's UI passes them.
    PA_SELECT_FOCAL_POINT, PA_SELECT_ACTIVE_VOXEL, PA_ADD_VOXEL, PA_REMOVE_VOXEL = range(4)

    def request_action(self, x: float, y: float, dx: float, dy: float, action: int, restart: bool = True):
        px, py = x * self.width, (1.0 - y) * self.height
        vx, vy = dx * self.width, -(dy * self.height)     # the add service flips the motion's y
        if action == self.PA_SELECT_FOCAL_POINT:
            if restart:
                self.job.reset()
            return self.pick_focal_distance(px, py)
        if action == self.PA_SELECT_ACTIVE_VOXEL:
            voxel, normal = self.job.select_voxel(px, py)
            if voxel[0] >= 0:
                self._settings.selected_voxel[:] = list(voxel)
                self.update_render_settings()
            return voxel, normal
        if action == self.PA_ADD_VOXEL:
            return self.job.add_voxel(px, py, vx, vy, restart)
        if action == self.PA_REMOVE_VOXEL:
            return self.job.remove_voxel(px, py, restart)
        raise ValueError(f"unknown action {action}")

    # Renderer::requestAction with the focal-distance service
    def pick_focal_distance(self, x: float, y: float):
        dist, voxel = self.job.pick(x, y)
        self._camera.focal_distance = dist
        self.update_camera()
        return dist, voxel

    def close(self):
        for o in (self.job, self.scene, self.env):
            if o:
                o.close()
        self.job = self.scene = self.env = None
        if self.ctx:
            self.ctx.close()
            self.ctx = None
