"""File ingest and image I/O through the library's host decoders (no GPU):
MagicaVoxel .vox (magicaVoxel.cpp:122-321 semantics), Wavefront OBJ
(meshLoader.cpp:11-74: all shapes merged, polygons fanned), PFM and
Radiance HDR.  Inputs are written by the tests from the published formats."""
import math
import os
import struct

import numpy as np
import pytest

from voxeltoy_gb300 import _lib as L
from voxeltoy_gb300 import formats as F


def chunk(tag: bytes, content: bytes, children: bytes = b"") -> bytes:
    return tag + struct.pack("<ii", len(content), len(children)) + content + children


def vox_file(size, voxels, rgba=None, version=150, extra=b""):
    kids = chunk(b"SIZE", struct.pack("<iii", *size))
    kids += chunk(b"XYZI", struct.pack("<i", len(voxels)) + b"".join(bytes(v) for v in voxels))
    kids += extra
    if rgba is not None:
        kids += chunk(b"RGBA", bytes(np.asarray(rgba, np.uint8).ravel()))
    return b"VOX " + struct.pack("<i", version) + chunk(b"MAIN", b"", kids)


def test_vox_axes_palette_order_and_empty_index():
    rgba = np.zeros((256, 4), np.uint8)
    rgba[:, 0] = np.arange(256)             # file entry i is colour index i + 1
    rgba[:, 1] = 255 - np.arange(256)
    rgba[:, 2] = 7
    rgba[:, 3] = 255
    vox = [(0, 0, 0, 9), (3, 2, 1, 4), (1, 1, 0, 9), (2, 0, 1, 254)]   # index 254 stays empty
    data = vox_file((4, 3, 2), vox, rgba, extra=chunk(b"nTRN", b"\x00" * 12))
    grid, pal = F.vox_decode(data)
    assert grid.shape == (3, 2, 4)          # [z, y, x] with res = (x, file z, file y)
    # file (x, y, z) -> (x, z, y): entries numbered by first use, 9 -> 1, 4 -> 2
    assert grid[0, 0, 0] == 1 and grid[2, 1, 3] == 2 and grid[1, 0, 1] == 1
    assert np.count_nonzero(grid) == 3
    assert len(pal) == 2
    t, e, a, r = pal[0]
    assert t == L.VT_MATERIAL_LAMBERT and e == (0.0, 0.0, 0.0)
    np.testing.assert_allclose(a, [8 / 255, 247 / 255, 7 / 255], rtol=1e-6)
    np.testing.assert_allclose(pal[1][2], [3 / 255, 252 / 255, 7 / 255], rtol=1e-6)


def test_vox_default_palette_and_versions():
    vox = [(0, 0, 0, 1), (1, 0, 0, 2), (0, 1, 0, 216), (1, 1, 0, 255), (0, 0, 1, 36)]
    grid, pal = F.vox_decode(vox_file((2, 2, 2), vox, version=200))
    cols = [tuple(round(c * 255) for c in p[2]) for p in pal]
    # the 6x6x6 cube (red slowest, blue fastest) then the red/green/blue/grey ramps
    assert cols == [(255, 255, 255), (255, 255, 204), (238, 0, 0), (17, 17, 17), (255, 0, 0)]
    with pytest.raises(L.VtError):
        F.vox_decode(vox_file((2, 2, 2), vox, version=151))
    with pytest.raises(L.VtError):
        F.vox_decode(vox_file((2, 2, 2), [(2, 0, 0, 1)]))          # outside the model
    with pytest.raises(L.VtError):
        F.vox_decode(b"VOX " + struct.pack("<i", 150))              # truncated


# The reference's sample inputs, found through VOXELTOY_REFERENCE_RESOURCES
# (its resources/ directory); the tests skip when that is unset or absent.
REF_RESOURCES = os.environ.get("VOXELTOY_REFERENCE_RESOURCES", "")
REF_VOX = os.path.join(REF_RESOURCES, "scene_fall.vox") if REF_RESOURCES else ""


@pytest.mark.skipif(not REF_VOX or not os.path.exists(REF_VOX),
                    reason="VOXELTOY_REFERENCE_RESOURCES does not point at the reference's sample scene")
def test_vox_reference_sample_scene():
    data = open(REF_VOX, "rb").read()
    grid, pal = F.vox_decode(data)
    # count the file's voxels independently
    pos, n_vox, size = 20 + struct.unpack_from("<i", data, 12)[0], 0, None
    while pos + 12 <= len(data):
        tag = data[pos:pos + 4]
        content, children = struct.unpack_from("<ii", data, pos + 4)
        if tag == b"SIZE":
            size = struct.unpack_from("<iii", data, pos + 12)
        if tag == b"XYZI":
            n = struct.unpack_from("<i", data, pos + 12)[0]
            xyzi = np.frombuffer(data, np.uint8, 4 * n, pos + 16).reshape(n, 4)
            n_vox = int(np.count_nonzero(xyzi[:, 3] != 254))
        pos += 12 + content + children
    assert grid.shape == (size[1], size[2], size[0])
    assert np.count_nonzero(grid) == n_vox and 0 < len(pal) <= 255


def test_obj_decode_faces_and_errors():
    text = """# a quad and a triangle
o first
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vn 0 0 1
f 1/1/1 2/1/1 3/1/1 4/1/1
v 0 0 2
f -3 -2 -1
g other
f 1//1 3//1 5//1
"""
    v, i = F.obj_decode(text)
    assert v.shape == (5, 3) and v[4].tolist() == [0, 0, 2]
    assert i.tolist() == [[0, 1, 2], [0, 2, 3], [2, 3, 4], [0, 2, 4]]
    for bad in ("v 0 0 0\nf 1 2 3\n", "v 0 0 0\nv 1 0 0\nf 1 2\n", "v 0 0\n"):
        with pytest.raises(L.VtError):
            F.obj_decode(bad)


def test_pfm_round_trip_and_variants():
    rng = np.random.default_rng(0)
    img = rng.normal(size=(5, 7, 4)).astype(np.float32)     # rows bottom first
    data = F.encode_pfm(img)
    assert data.startswith(b"PF\n7 5\n-1.0\n")
    np.testing.assert_array_equal(F.image_decode(data), img[::-1, :, :3])   # decoded rows top first
    # big-endian colour and grey PFMs written by hand
    be = img[..., :3].astype(">f4")
    np.testing.assert_array_equal(F.image_decode(b"PF\n7 5\n1.0\n" + be.tobytes()), img[::-1, :, :3])
    g = img[..., 0].astype("<f4")
    got = F.image_decode(b"Pf\n7 5\n-1.0\n" + g.tobytes())
    np.testing.assert_array_equal(got, np.repeat(img[::-1, :, :1], 3, axis=2))
    with pytest.raises(L.VtError):
        F.image_decode(b"PF\n7 5\n-1.0\n" + be.tobytes()[:-4])


def rgbe(rgb):
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    m = rgb.max(axis=-1)
    nz = m > 1e-32
    e = np.zeros(m.shape, np.int64)
    f, e[nz] = np.frexp(m[nz])
    scale = np.zeros(m.shape)
    scale[nz] = 256.0 / np.ldexp(1.0, e[nz])
    out[..., :3] = np.clip(np.floor(rgb * scale[..., None]), 0, 255).astype(np.uint8)
    out[..., 3] = np.where(nz, e + 128, 0)
    return out


def expected_from_rgbe(q):
    m = q[..., :3].astype(np.float64) + 0.5
    ex = q[..., 3].astype(np.int64)
    val = np.ldexp(m, (ex - 136)[..., None])
    return np.where((ex == 0)[..., None], 0.0, val).astype(np.float32)


def rle_scanline(q):
    """New-style run-length scanline: 2 2 w_hi w_lo, then four channel planes."""
    w = q.shape[0]
    out = bytearray([2, 2, w >> 8, w & 255])
    for c in range(4):
        plane = q[:, c]
        x = 0
        while x < w:
            run = 1
            while x + run < w and run < 127 and plane[x + run] == plane[x]:
                run += 1
            if run >= 3:
                out += bytes([128 + run, plane[x]])
                x += run
            else:
                lit = min(128, w - x)
                # literal until the next run of 3
                k = 0
                while k < lit:
                    if k + 2 < lit and plane[x + k] == plane[x + k + 1] == plane[x + k + 2]:
                        break
                    k += 1
                k = max(k, 1)
                out += bytes([k]) + bytes(plane[x:x + k])
                x += k
    return bytes(out)


def test_radiance_hdr_flat_and_rle():
    rng = np.random.default_rng(1)
    w, h = 40, 6
    rgb = np.exp(rng.normal(0, 3, (h, w, 3)))
    rgb[2, 5:20] = 0.25                              # runs for the RLE encoder
    q = rgbe(rgb)
    head = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n" + f"-Y {h} +X {w}\n".encode()
    flat = head + q.tobytes()
    want = expected_from_rgbe(q)
    np.testing.assert_array_equal(F.image_decode(flat), want)
    rle = head + b"".join(rle_scanline(q[y]) for y in range(h))
    np.testing.assert_array_equal(F.image_decode(rle), want)
    # RGBE keeps 8 bits of mantissa under the pixel's largest channel
    assert np.all(np.abs(want - rgb) <= rgb.max(axis=-1, keepdims=True) / 128)
    with pytest.raises(L.VtError):
        F.image_decode(b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 1 +X 1\n\x00\x00\x00\x00")


REF_OBJ = os.path.join(REF_RESOURCES, "bunny.obj") if REF_RESOURCES else ""


@pytest.mark.skipif(not REF_OBJ or not os.path.exists(REF_OBJ),
                    reason="VOXELTOY_REFERENCE_RESOURCES does not point at the reference's sample mesh")
def test_obj_reference_sample_mesh():
    v, i = F.obj_decode(REF_OBJ)
    assert len(v) > 1000 and len(i) > 1000
    assert i.max() < len(v) and np.isfinite(v).all()


def test_hdr_encode_round_trip():
    """vt_image_encode_hdr: rows bottom first in, top first in the file (the
    decoder returns them top first), RGBE precision (8 bits of mantissa under
    the largest channel), zeros, and negative / NaN / infinite channels."""
    rng = np.random.default_rng(8)
    h, w = 7, 11
    img = (rng.random((h, w, 4)) * np.exp2(rng.integers(-10, 12, (h, w, 1)))).astype(np.float32)
    img[0, 0, :3] = 0.0
    img[1, 2, :3] = [-1.0, np.nan, 2.0]
    img[2, 3, :3] = [np.inf, 1.0, 0.5]
    data = F.encode_hdr(img)
    assert data.startswith(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 7 +X 11\n")
    got = F.image_decode(data)[::-1]                       # back to rows bottom first
    rgb = np.nan_to_num(np.clip(img[..., :3], 0.0, None), nan=0.0, posinf=1.0e38).astype(np.float64)
    ok = np.ones((h, w), bool)
    ok[2, 3] = False
    scale = rgb.max(axis=-1, keepdims=True)
    assert np.all(np.abs(got - rgb)[ok] <= (scale / 128)[ok] + 1e-30)
    assert np.all(got[0, 0] == 0.0)
    # a zero mantissa beside a larger channel reads back as half a quantum of that channel
    assert got[1, 2, 0] <= 2.0 / 256 and got[1, 2, 1] <= 2.0 / 256 and abs(got[1, 2, 2] - 2.0) <= 2.0 / 128
    assert got[2, 3, 0] > 0.99e38
