"""File formats on the path's edges, through the library's decoders (no GPU
needed): MagicaVoxel .vox, Wavefront OBJ, PFM and Radiance HDR images."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _bytes(data) -> bytes:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return bytes(data)
    with open(data, "rb") as f:
        return f.read()


def vox_decode(data):
    """.vox bytes or path -> (voxels uint8 [z, y, x], palette tuples)."""
    b = _bytes(data)
    res = (C.c_int32 * 3)()
    n = C.c_int32()
    L.call("vt_vox_decode", b, len(b), res, None, 0, None, C.byref(n))
    rx, ry, rz = res
    vox = np.empty((rz, ry, rx), np.uint8)
    pal = (L.Material * max(1, n.value))()
    L.call("vt_vox_decode", b, len(b), res, L.ptr(vox), vox.nbytes, pal, C.byref(n))
    palette = [(m.type, tuple(m.emission), tuple(m.albedo), m.roughness) for m in pal[: n.value]]
    return vox, palette


def obj_decode(text):
    """OBJ text (str/bytes) or path -> (vertices float32 [n, 3], indices uint32 [t, 3])."""
    # a str with a line break is OBJ text, any other str a path
    b = text.encode() if isinstance(text, str) and "\n" in text else _bytes(text)
    nv, nt = C.c_int64(), C.c_int64()
    L.call("vt_obj_decode", b, len(b), None, 0, None, 0, C.byref(nv), C.byref(nt))
    v = np.empty((nv.value, 3), np.float32)
    i = np.empty((nt.value, 3), np.uint32)
    L.call("vt_obj_decode", b, len(b), L.ptr(v), nv.value, L.ptr(i), nt.value, C.byref(nv), C.byref(nt))
    return v, i


def image_decode(data) -> np.ndarray:
    """PFM or Radiance HDR bytes or path -> float32 [h, w, 3], rows top first."""
    b = _bytes(data)
    w, h = C.c_int32(), C.c_int32()
    L.call("vt_image_decode", b, len(b), None, 0, C.byref(w), C.byref(h))
    out = np.empty((h.value, w.value, 3), np.float32)
    L.call("vt_image_decode", b, len(b), L.ptr(out), out.nbytes, C.byref(w), C.byref(h))
    return out


def encode_pfm(pixels: np.ndarray) -> bytes:
    """float [h, w, 3 or 4], rows bottom first (vt_job_readback's order) -> PFM bytes."""
    px = np.ascontiguousarray(pixels, dtype=np.float32)
    h, w, ch = px.shape
    n = C.c_size_t()
    L.call("vt_image_encode_pfm", L.ptr(px), w, h, ch, None, 0, C.byref(n))
    out = (C.c_uint8 * n.value)()
    L.call("vt_image_encode_pfm", L.ptr(px), w, h, ch, out, n.value, C.byref(n))
    return bytes(out)


def encode_hdr(pixels: np.ndarray) -> bytes:
    """float [h, w, 3 or 4], rows bottom first (vt_job_readback's order) ->
    Radiance RGBE bytes (rows top first in the file)."""
    px = np.ascontiguousarray(pixels, dtype=np.float32)
    h, w, ch = px.shape
    n = C.c_size_t()
    L.call("vt_image_encode_hdr", L.ptr(px), w, h, ch, None, 0, C.byref(n))
    out = (C.c_uint8 * n.value)()
    L.call("vt_image_encode_hdr", L.ptr(px), w, h, ch, out, n.value, C.byref(n))
    return bytes(out)
