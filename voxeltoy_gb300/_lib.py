"""ctypes binding of libvoxeltoy.so (include/vt.h and include/vt_diag.h).

The structures mirror the C declarations field for field.  Loading the
library needs no GPU; every call that touches the device fails with
VT_EDEVICE when none is present.  The library must exist: there is no
Python or CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

VT_OK, VT_EINVAL, VT_ENOMEM, VT_EBUDGET, VT_EDEVICE, VT_ETIMEOUT, VT_ECANCELLED, VT_ENOTREADY, VT_EUNSUPPORTED = (
    0, -1, -2, -3, -4, -5, -6, -7, -8)
VT_SAMPLES_PENDING, VT_FINISHED_RENDERING = 0, 1
VT_MATERIAL_LAMBERT, VT_MATERIAL_METAL, VT_MATERIAL_PLASTIC = 0, 1, 2
VT_SCENE_PRUNE_EMISSIVE, VT_SCENE_AUTO_EMISSIVE = 1, 2
VT_VOXELIZE_THIN, VT_VOXELIZE_FAT, VT_VOXELIZE_REFERENCE_BOUNDS = 0, 1, 0x100
VT_MESH_VOXEL_SPACE, VT_MESH_FIT_UNIT_CUBE = 0, 1
VT_LENS_PINHOLE, VT_LENS_THIN_LENS, VT_LENS_ORTHOGRAPHIC = 0, 1, 2
VT_SERVE_ARRIVAL, VT_SERVE_LEAST_WORK = 0, 1
VT_ENV_CDF_REFERENCE_SIZE = 1
VT_DEVICE_NO_ALLOC_CACHE = 1
VT_INTEGRATOR_PATH_TRACER, VT_INTEGRATOR_EDIT_MODE = 0, 1
VT_BUTTON_ROTATE, VT_BUTTON_PAN = 1, 2
VT_KEY_FORWARD, VT_KEY_BACK, VT_KEY_RIGHT, VT_KEY_LEFT = 0, 1, 2, 3
VT_QUIRK_GAMMA_BEFORE_AVERAGE = 1 << 0
VT_QUIRK_GROUND = 1 << 1
VT_QUIRK_GRADIENT_PDF_MISMATCH = 1 << 2
VT_QUIRK_DOUBLE_REFLECTANCE = 1 << 3
VT_QUIRK_FIXED_IOR = 1 << 4
VT_QUIRK_EXPONENT_IS_ROUGHNESS = 1 << 5
VT_QUIRK_THINLENS_NO_JITTER = 1 << 6
VT_QUIRK_UNGUARDED_SAMPLES = 1 << 7
VT_QUIRKS_REFERENCE = 0xFF
VT_RNG_PHILOX, VT_RNG_NOISE_TABLE = 0, 1
VT_READBACK_FLIP_Y, VT_READBACK_TONEMAP = 1, 2
VT_REQ_QUEUED, VT_REQ_RUNNING, VT_REQ_DONE, VT_REQ_CANCELLED, VT_REQ_FAILED = 0, 1, 2, 3, 4
VT_DIAG_NUM_COUNTERS = 9

f3 = C.c_float * 3
i3 = C.c_int32 * 3


class DeviceOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("hbm_budget_bytes", C.c_uint64), ("flags", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("emission", f3), ("albedo", f3), ("roughness", C.c_float)]


class SceneInfo(C.Structure):
    _fields_ = [("resolution", i3), ("bounds_min", f3), ("bounds_max", f3), ("voxel_size", f3),
                ("n_emissive", C.c_int64), ("n_palette", C.c_int32), ("device_bytes", C.c_uint64)]


class Camera(C.Structure):
    _fields_ = [("eye", f3), ("target", f3), ("fov_y", C.c_float), ("near_distance", C.c_float),
                ("far_distance", C.c_float), ("focal_distance", C.c_float), ("lens_radius", C.c_float),
                ("lens_model", C.c_int32)]


class CameraUniforms(C.Structure):
    _fields_ = [("proj", C.c_float * 16), ("inv_proj", C.c_float * 16), ("inv_model_view", C.c_float * 16),
                ("viewport", C.c_float * 4)]


class RenderSettings(C.Structure):
    _fields_ = [("max_bounces", C.c_int32), ("max_samples", C.c_int32), ("rr_start_bounce", C.c_int32),
                ("gamma", C.c_float), ("exposure", C.c_float), ("nee_emission_scale", C.c_float),
                ("wireframe_opacity", C.c_float), ("wireframe_thickness", C.c_float),
                ("background_top", f3), ("background_bottom", f3), ("background_rotation", C.c_float),
                ("selected_voxel", i3), ("select_enabled", C.c_int32), ("ground_material", C.c_int32),
                ("quirks", C.c_uint32), ("rng_mode", C.c_int32), ("seed", C.c_uint32)]


class BatchOpts(C.Structure):
    _fields_ = [("path_slots", C.c_int32), ("blocks_per_sm", C.c_int32), ("threads_per_block", C.c_int32),
                ("kernel", C.c_int32)]


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_active_jobs", C.c_int32), ("passes_per_round", C.c_int32),
                ("path_slots", C.c_int32), ("order", C.c_int32), ("quick_paths", C.c_uint64),
                ("round_paths_cap", C.c_uint64), ("round_paths", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("cancelled", C.c_uint64),
                ("failed", C.c_uint64), ("paths_traced", C.c_uint64), ("rounds", C.c_uint64),
                ("bytes_in_use", C.c_uint64), ("active", C.c_int32), ("queued", C.c_int32),
                ("scene_uploads", C.c_uint64), ("scene_hits", C.c_uint64), ("scene_evictions", C.c_uint64),
                ("scenes_resident", C.c_int32), ("pad", C.c_int32), ("round_us", C.c_uint64),
                ("between_us", C.c_uint64)]


P = C.c_void_p
PP = C.POINTER(C.c_void_p)
fp = C.POINTER(C.c_float)
LOG_FN = C.CFUNCTYPE(None, C.c_char_p, C.c_void_p)

# name -> (argtypes) ; every function returns int
SIGNATURES = {
    "vt_create": [C.POINTER(DeviceOpts), PP],
    "vt_destroy": [P],
    "vt_set_log_callback": [P, LOG_FN, P],
    "vt_context_memory": [P, C.POINTER(C.c_uint64)],
    "vt_context_trim": [P, C.POINTER(C.c_uint64)],
    "vt_scene_create": [P, C.c_int32, C.c_int32, C.c_int32, P, C.POINTER(Material), C.c_int32, P, C.c_int64,
                        C.c_uint32, PP],
    "vt_scene_create_from_offsets": [P, C.c_int32, C.c_int32, C.c_int32, P, P, C.c_int64, P, C.c_int64, C.c_uint32,
                                     PP],
    "vt_scene_voxelize_mesh": [P, P, C.c_int64, P, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                               C.POINTER(Material), C.c_int32, PP],
    "vt_scene_get_info": [P, C.POINTER(SceneInfo)],
    "vt_scene_read_voxels": [P, P, C.c_size_t],
    "vt_scene_read_emissive": [P, P, C.c_int64, C.POINTER(C.c_int64)],
    "vt_scene_read_material_table": [P, P, C.c_int64, C.POINTER(C.c_int64)],
    "vt_scene_write_material_table": [P, C.c_int64, P, C.c_int32],
    "vt_scene_destroy": [P],
    "vt_scene_set_brick_shape": [P, C.c_int32, C.c_int32, C.c_int32],
    "vt_scene_get_brick_shape": [P, C.POINTER(C.c_int32)],
    "vt_env_create_image": [P, P, C.c_int32, C.c_int32, PP],
    "vt_env_create_image_ex": [P, P, C.c_int32, C.c_int32, C.c_uint32, PP],
    "vt_env_get_info": [P, C.POINTER(C.c_int32)],
    "vt_env_read_cdf": [P, P, C.c_size_t, P, C.c_size_t, fp],
    "vt_env_destroy": [P],
    "vt_camera_default": [C.POINTER(Camera)],
    "vt_camera_orbit": [C.POINTER(Camera), C.c_float, C.c_float],
    "vt_camera_orbit_eye": [C.POINTER(Camera), C.c_float, C.c_float],
    "vt_camera_set_distance": [C.POINTER(Camera), C.c_float],
    "vt_camera_set_focal_length": [C.POINTER(Camera), C.c_float, C.c_int32, C.c_int32],
    "vt_camera_set_fstop": [C.POINTER(Camera), C.c_float, C.c_int32, C.c_int32],
    "vt_camera_focus_on_bounds": [C.POINTER(Camera), fp, fp],
    "vt_camera_orbit_mouse": [C.POINTER(Camera), C.c_float, C.c_float, C.c_int32],
    "vt_camera_fly_mouse": [C.POINTER(Camera), C.c_float, C.c_float, C.c_int32],
    "vt_camera_fly_key": [C.POINTER(Camera), C.c_int32],
    "vt_camera_compute_uniforms": [C.POINTER(Camera), C.c_int32, C.c_int32, C.POINTER(CameraUniforms)],
    "vt_settings_default": [C.POINTER(RenderSettings)],
    "vt_job_create": [P, P, P, C.POINTER(Camera), C.POINTER(RenderSettings), C.c_int32, C.c_int32, PP],
    "vt_job_set_camera": [P, C.POINTER(Camera)],
    "vt_job_set_settings": [P, C.POINTER(RenderSettings)],
    "vt_job_set_scene": [P, P, P],
    "vt_job_resize": [P, C.c_int32, C.c_int32],
    "vt_job_reset": [P],
    "vt_job_set_integrator": [P, C.c_int32],
    "vt_job_render": [P, C.c_int32, C.POINTER(C.c_int32)],
    "vt_job_synchronize": [P],
    "vt_job_sample_count": [P, C.POINTER(C.c_int32)],
    "vt_job_readback": [P, P, C.c_size_t, C.c_uint32],
    "vt_job_device_buffer": [P, PP, C.POINTER(C.c_int32)],
    "vt_job_snapshot": [P, P, P, C.c_size_t, C.POINTER(C.c_int32)],
    "vt_job_restore": [P, P, P, C.c_size_t, C.c_int32],
    "vt_job_pick": [P, C.c_float, C.c_float, fp, C.POINTER(C.c_int32)],
    "vt_job_destroy": [P],
    "vt_render_batch": [P, C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.POINTER(BatchOpts), C.POINTER(C.c_int32)],
    "vt_render_batch_fixed": [P, C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)],
    "vt_vox_decode": [P, C.c_size_t, C.POINTER(C.c_int32), P, C.c_size_t, P, C.POINTER(C.c_int32)],
    "vt_scene_set_voxel": [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32],
    "vt_job_select_voxel": [P, C.c_float, C.c_float, C.POINTER(C.c_int32), fp],
    "vt_job_add_voxel": [P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32, C.POINTER(C.c_int32)],
    "vt_job_remove_voxel": [P, C.c_float, C.c_float, C.c_int32, C.POINTER(C.c_int32)],
    "vt_scene_create_from_vox": [P, P, C.c_size_t, C.c_uint32, PP],
    "vt_obj_decode": [P, C.c_size_t, P, C.c_int64, P, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
    "vt_scene_voxelize_obj": [P, P, C.c_size_t, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32,
                              PP],
    "vt_image_decode": [P, C.c_size_t, P, C.c_size_t, C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
    "vt_image_encode_pfm": [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_size_t, C.POINTER(C.c_size_t)],
    "vt_image_encode_hdr": [P, C.c_int32, C.c_int32, C.c_int32, P, C.c_size_t, C.POINTER(C.c_size_t)],
    "vt_server_create": [P, C.POINTER(ServerOpts), PP],
    "vt_server_submit": [P, P, P, C.POINTER(Camera), C.POINTER(RenderSettings), C.c_int32, C.c_int32, C.c_int32,
                         C.POINTER(C.c_uint64)],
    "vt_server_submit_dense": [P, C.c_uint64, C.c_int32, C.c_int32, C.c_int32, P, C.POINTER(Material), C.c_int32,
                               C.c_uint32, P, C.POINTER(Camera), C.POINTER(RenderSettings), C.c_int32, C.c_int32,
                               C.c_int32, C.POINTER(C.c_uint64)],
    "vt_server_poll": [P, C.c_uint64, C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
    "vt_server_wait": [P, C.c_uint64, C.c_double],
    "vt_server_result": [P, C.c_uint64, P, C.c_size_t, C.POINTER(C.c_double)],
    "vt_server_cancel": [P, C.c_uint64],
    "vt_server_get_stats": [P, C.POINTER(ServerStats)],
    "vt_server_destroy": [P],
    "vt_diag_trace_rays": [P, P, P, C.c_int64, P],
    "vt_diag_samples": [P, C.c_int32, P, P, P],
    "vt_diag_render_counted": [P, C.c_int32, P, C.POINTER(C.c_int32)],
    "vt_diag_set_kernel": [P, C.c_int32],
    "vt_diag_set_graphs": [P, C.c_int32],
    "vt_diag_set_lanes": [P, C.c_int32],
    "vt_diag_builtins": [P, C.c_int32, P, P, P, C.c_int64],
    "vt_diag_cdf_from_function": [P, P, C.c_int32, C.c_int32, P, P, fp],
    "vt_diag_env_texels": [P, P, C.c_size_t],
    "vt_diag_stream": [P, PP],
    "vt_diag_launch_count": [P, C.POINTER(C.c_uint64)],
    "vt_diag_l2_read_bandwidth": [P, C.c_int64, C.c_int32, C.POINTER(C.c_double)],
    "vt_diag_check_word": [P, C.POINTER(C.c_uint32), C.POINTER(C.c_int32)],
    "vt_diag_scene_bricks": [P, P, C.c_size_t, C.POINTER(C.c_int64)],
    "vt_diag_set_tuning": [P, C.c_int64, C.c_int32, C.c_int32, C.c_int64],
    "vt_diag_set_trace_tuning": [P, C.c_int32, C.c_int32],
    "vt_diag_set_trace_form": [P, C.c_int32],
    "vt_diag_set_noise_table": [P, P, C.c_size_t],
    "vt_diag_get_noise_table": [P, P, C.c_size_t],
}

_LIB = None


class VtError(RuntimeError):
    def __init__(self, code: int, fn: str, msg: str):
        super().__init__(f"{fn} failed with {code}: {msg}")
        self.code = code


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libvoxeltoy.so (building it first if it is missing or stale);
    with VOXELTOY_CHECKED=1 in the environment, the bounds-checked build
    libvoxeltoy_checked.so instead."""
    global _LIB
    if _LIB is not None:
        return _LIB
    import os
    checked = os.environ.get("VOXELTOY_CHECKED") == "1"
    path = _build.CHECKED_LIB if checked else _build.LIB
    if build_if_missing and not _build.up_to_date(checked):
        _build.build(checked=checked)
    if not Path(path).exists():
        raise RuntimeError(f"{path} is missing: run voxeltoy_gb300.build.build()")
    lib = C.CDLL(str(path))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.vt_last_error.argtypes = []
    lib.vt_last_error.restype = C.c_char_p
    _LIB = lib
    return lib


def check(rc: int, fn: str = "vt call") -> int:
    if rc != VT_OK:
        msg = load().vt_last_error().decode(errors="replace")
        raise VtError(rc, fn, msg)
    return rc


def call(name: str, *args) -> int:
    return check(getattr(load(), name)(*args), name)


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return C.c_void_p(a.ctypes.data)


def materials(records) -> C.Array:
    """Array of Material from (type, emission, albedo, roughness) tuples or dicts."""
    arr = (Material * max(1, len(records)))()
    for i, r in enumerate(records):
        if isinstance(r, dict):
            r = (r["type"], r.get("emission", (0, 0, 0)), r.get("albedo", (0, 0, 0)), r.get("roughness", 0.0))
        t, e, a, rough = r
        arr[i].type = int(t)
        arr[i].emission[:] = [float(x) for x in e]
        arr[i].albedo[:] = [float(x) for x in a]
        arr[i].roughness = float(rough)
    return arr
