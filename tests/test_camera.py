"""Camera math of the host runtime (Renderer::updateCamera and the camera
controllers) against the oracle and against float64 restatements.  These
entry points are pure host code and run without a GPU."""
import ctypes as C
import math

import numpy as np
import pytest

from voxeltoy_gb300 import _lib as L
from voxeltoy_gb300 import camera_uniforms, default_camera


def make_cam(eye, target, fov_deg=45.0, lens=0):
    cam = default_camera()
    cam.eye[:] = eye
    cam.target[:] = target
    cam.fov_y = math.radians(fov_deg)
    cam.lens_model = lens
    return cam


CASES = [
    ((0, 0, -100), (0, 0, 0), 45.0, 0, 256, 256),
    ((1224.7, 1000.0, -1224.7), (0, 0, 0), 45.0, 0, 320, 200),
    ((-300, 800, 650), (10, -20, 30), 30.0, 1, 200, 320),
    ((500, 500, 500), (0, 0, 0), 60.0, 2, 640, 480),
]


@pytest.mark.parametrize("eye,target,fov,lens,w,h", CASES)
def test_uniforms_match_oracle_bitwise(orc, eye, target, fov, lens, w, h):
    cam = make_cam(eye, target, fov, lens)
    u = camera_uniforms(cam, w, h)
    ref = orc.camera_uniforms(cam, w, h)
    np.testing.assert_array_equal(u["proj"], ref[0:16])
    np.testing.assert_array_equal(u["inv_proj"], ref[16:32])
    np.testing.assert_array_equal(u["inv_model_view"], ref[32:48])
    np.testing.assert_array_equal(u["viewport"], ref[48:52])


@pytest.mark.parametrize("eye,target,fov,lens,w,h", CASES)
def test_uniforms_match_gl_math(eye, target, fov, lens, w, h):
    """gluLookAt / gluPerspective / gluOrtho2D in float64 (renderer.cpp:355-394)."""
    cam = make_cam(eye, target, fov, lens)
    u = camera_uniforms(cam, w, h)
    e, t = np.array(eye, float), np.array(target, float)
    f = (t - e) / np.linalg.norm(t - e)
    r = np.cross([0, 1, 0], f)
    r /= np.linalg.norm(r)
    up = np.cross(f, r)
    mv = np.eye(4)
    mv[0, :3], mv[1, :3], mv[2, :3] = r, up, -f
    mv[:3, 3] = [-e @ r, -e @ up, e @ f]
    a = w / h
    fy = math.radians(fov)
    if lens == 2:
        dist = np.linalg.norm(t - e)
        left = -math.tan(fy / 2) * dist
        bottom = left / a
        n, fr = -0.1, -10000.0
        pm = np.diag([2 / (-2 * left), 2 / (-2 * bottom), -2 / (fr - n), 1.0])
        pm[2, 3] = -(fr + n) / (fr - n)
    else:
        ee = 1 / math.tan(fy / 2)
        n, fr = 0.1, 10000.0
        pm = np.zeros((4, 4))
        pm[0, 0], pm[1, 1] = ee / a, ee
        pm[2, 2], pm[2, 3], pm[3, 2] = (fr + n) / (n - fr), 2 * fr * n / (n - fr), -1
    np.testing.assert_allclose(u["proj"].reshape(4, 4), pm, rtol=2e-6, atol=1e-9)
    np.testing.assert_allclose(u["inv_model_view"].reshape(4, 4), np.linalg.inv(mv), rtol=1e-5, atol=2e-4)
    np.testing.assert_allclose(u["inv_proj"].reshape(4, 4), np.linalg.inv(pm), rtol=1e-4, atol=1e-6)


def test_orbit_and_distance():
    cam = make_cam((0, 0, -2000), (0, 0, 0))
    L.call("vt_camera_orbit", C.byref(cam), math.radians(120), math.radians(45))
    th, ph = math.radians(120), math.radians(45)
    want = -2000 * np.array([math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph)])
    np.testing.assert_allclose(list(cam.eye), want, rtol=1e-5)
    L.call("vt_camera_set_distance", C.byref(cam), 500.0)
    assert np.linalg.norm(np.array(cam.eye) - np.array(cam.target)) == pytest.approx(500.0, rel=1e-5)


def test_focal_length_and_fstop():
    cam = default_camera()
    # setFocalLength(50) with 36 mm film: fov = 2 atan(18 / 50)
    assert cam.fov_y == pytest.approx(2 * math.atan(18 / 50), rel=1e-6)
    L.call("vt_camera_set_focal_length", C.byref(cam), 35.0, 300, 200)   # landscape: film 36 x 24
    assert cam.fov_y == pytest.approx(2 * math.atan(12 / 35), rel=1e-6)
    L.call("vt_camera_set_fstop", C.byref(cam), 2.0, 300, 200)
    assert cam.lens_radius == pytest.approx(35.0 / 2.0 * 0.5, rel=1e-5)


def test_focus_on_bounds_and_fly():
    cam = make_cam((0, 0, -10), (0, 0, 0), 45.0)
    bmin = (C.c_float * 3)(-500, -250, -500)
    bmax = (C.c_float * 3)(500, 250, 500)
    L.call("vt_camera_focus_on_bounds", C.byref(cam), bmin, bmax)
    d = math.sqrt(1000 ** 2 + 500 ** 2 + 1000 ** 2) / (2 * math.tan(math.radians(45) / 2))
    np.testing.assert_allclose(list(cam.eye), [0, 0, -d], rtol=1e-5)
    before = np.array(cam.eye)
    L.call("vt_camera_fly_key", C.byref(cam), L.VT_KEY_FORWARD)
    np.testing.assert_allclose(np.array(cam.eye) - before, [0, 0, 100], atol=1e-3)
    L.call("vt_camera_fly_key", C.byref(cam), L.VT_KEY_RIGHT)
    # right = Y x forward = (1, 0, 0) x ... for forward +Z: (0,1,0) x (0,0,1) = (1, 0, 0)
    np.testing.assert_allclose(np.array(cam.eye) - before, [100, 0, 100], atol=1e-3)
    with pytest.raises(L.VtError):
        L.call("vt_camera_fly_key", C.byref(cam), 9)
