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


def _frame(cam):
    """CameraParameters::getBasis (cameraParameters.cpp:43-50): forward to the
    target, right = (0, 1, 0) x forward, up = forward x right.  That right
    vector points to the viewer's left, so window x runs the other way from
    a gluLookAt frame: the reference's images are mirrored left to right."""
    eye = np.array(cam.eye, float)
    f = np.array(cam.target, float) - eye
    f /= np.linalg.norm(f)
    r = np.cross([0.0, 1.0, 0.0], f)
    r /= np.linalg.norm(r)
    return eye, f, r, np.cross(f, r)


def _pixel_dirs(cam, w, h, frag):
    """World direction through window position frag of a perspective camera
    with vertical field of view fov_y and aspect w / h."""
    eye, f, r, u = _frame(cam)
    t = math.tan(cam.fov_y / 2)
    nx = 2 * frag[:, 0] / w - 1
    ny = 2 * frag[:, 1] / h - 1
    d = f[None] + (nx * t * w / h)[:, None] * r[None] + (ny * t)[:, None] * u[None]
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def test_generated_rays_follow_the_camera_geometry(orc):
    """generateRay (generateRay.h:1-123) on the oracle, against the geometry it
    implements: a pinhole ray leaves the eye through the jittered pixel
    position; thin-lens rays for one window position leave the lens disk
    and all pass through one point on the focal plane; orthographic rays are
    parallel to the view axis."""
    from voxeltoy_gb300 import scenes as S
    rng = np.random.default_rng(8)
    w, h = 320, 200
    s = S.physical_settings(max_bounces=1)
    n = 2000
    frag = np.stack([rng.uniform(0, w, n), rng.uniform(0, h, n)], 1)
    u = rng.random((n, 4))
    # pinhole: jitter u - 0.5 in window units (generateRay.h:15-25)
    cam = make_cam((-300.0, 800.0, 650.0), (10.0, -20.0, 30.0), 40.0, L.VT_LENS_PINHOLE)
    o, d = orc.generate_rays(cam, s, w, h, frag, u)
    want = _pixel_dirs(cam, w, h, frag + (u[:, :2] - 0.5))
    assert np.abs(o - np.array(cam.eye)).max() < 1e-3
    assert np.linalg.norm(d - want, axis=1).max() < 2e-5
    # thin lens without jitter: the rays of one window position meet on the
    # focal plane, at focal_distance along the view axis
    cam = make_cam((0.0, 400.0, -1800.0), (0.0, 0.0, 0.0), 45.0, L.VT_LENS_THIN_LENS)
    cam.lens_radius, cam.focal_distance = 40.0, 1500.0
    s.quirks = L.VT_QUIRK_THINLENS_NO_JITTER
    eye, f, r, up = _frame(cam)
    for k in range(20):
        fr = np.repeat(frag[k:k + 1], 64, 0)
        o, d = orc.generate_rays(cam, s, w, h, fr, rng.random((64, 4)))
        o = o.astype(np.float64)
        d = d.astype(np.float64)
        off = o - eye
        assert np.abs(off @ f).max() < 1e-3                       # the lens lies in the eye plane
        assert np.linalg.norm(off, axis=1).max() <= 40.0 + 1e-3
        p = _pixel_dirs(cam, w, h, frag[k:k + 1])[0]
        focus = eye + p * (1500.0 / (p @ f))                      # on the plane at 1500 along the view axis
        t = ((focus - o) * d).sum(1)
        miss = np.linalg.norm(o + t[:, None] * d - focus, axis=1)
        assert miss.max() < 2e-2
    # orthographic: every ray parallel to the view axis
    cam = make_cam((500.0, 500.0, 500.0), (0.0, 0.0, 0.0), 60.0, L.VT_LENS_ORTHOGRAPHIC)
    s.quirks = 0
    o, d = orc.generate_rays(cam, s, w, h, frag, u)
    assert np.abs(d - _frame(cam)[1]).max() < 1e-6
    assert np.ptp((o - np.array(cam.eye)) @ _frame(cam)[1]) < 1e-2  # origins on one plane
