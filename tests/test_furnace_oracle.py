"""White furnace on the CPU oracle: the integrator's composition of
raygen, DDA, NEE with MIS, BSDF sampling and accumulation
(pathTracer.fs:64-296) against an analytic answer.

A convex object under a constant environment L = 1 with a Lambert albedo
rho reflects exactly rho in expectation; a pixel that sees only the
environment is exactly 1.  Checked with the gradient background (uniform
hemisphere light samples, pdf 1/2pi) and with a constant image (light
samples from the image's CDFs, pdf = luminance / integral = 1/4pi), both
with the pdf mismatch of the gradient mode corrected (quirks off)."""
import numpy as np
import pytest

from voxeltoy_gb300 import scenes as S

RHO = 0.6


def furnace_frame(orc, env_rgb):
    g = np.zeros((16, 16, 16), np.uint8)
    g[4:12, 4:12, 4:12] = 1
    sc = orc.Scene(g, [S.lambert(RHO)])
    env = orc.Env(env_rgb) if env_rgb is not None else orc.Env()
    s = S.physical_settings(max_bounces=4)
    cam = S.orbit_camera(distance=1800.0, theta_deg=110.0, phi_deg=30.0)
    w = h = 32
    hit_any = np.zeros((h, w), bool)
    hit_all = np.ones((h, w), bool)
    for k in range(6):
        _, hits, _ = orc.render_samples(cam, s, sc, env, w, h, k)
        m = ((hits[..., 3] >> 8) & 1).astype(bool)
        hit_any |= m
        hit_all &= m
    img, _ = orc.render_average(cam, s, sc, env, w, h, 96)
    # pixels whose whole 3x3 neighbourhood always / never hit (silhouettes excluded)
    pa = np.pad(hit_any, 1, constant_values=True)
    pl = np.pad(hit_all, 1, constant_values=False)
    never = np.ones((h, w), bool)
    always = np.ones((h, w), bool)
    for dy in range(3):
        for dx in range(3):
            never &= ~pa[dy:dy + h, dx:dx + w]
            always &= pl[dy:dy + h, dx:dx + w]
    return img[..., :3], never, always


@pytest.mark.parametrize("env", ["gradient", "image"])
def test_white_furnace_oracle(orc, env):
    rgb = None if env == "gradient" else np.ones((32, 64, 3), np.float32)
    img, never, always = furnace_frame(orc, rgb)
    assert never.sum() > 50 and always.sum() > 50
    np.testing.assert_allclose(img[never], 1.0, rtol=0, atol=1e-6)
    assert abs(img[always].mean() - RHO) < 0.01
