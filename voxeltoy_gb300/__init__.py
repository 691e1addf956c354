"""GB300-native voxel path tracer and mesh voxelizer (voxelToy's rendering path).

The compute path lives in libvoxeltoy.so (CUDA for sm_103a) behind the C ABI
declared in include/vt.h; this package builds it, binds it with ctypes and
mirrors the reference's Renderer interface.
"""
from . import _lib as lib
from .renderer import (RR_FINISHED_RENDERING, RR_SAMPLES_PENDING, Context, Env, Job, Renderer, Scene, Server,
                       camera_uniforms, default_camera, default_settings)

__all__ = ["lib", "Context", "Scene", "Env", "Job", "Server", "Renderer", "default_camera", "default_settings",
           "camera_uniforms", "RR_SAMPLES_PENDING", "RR_FINISHED_RENDERING"]
