"""Known answers for the oracle's BSDFs and environment light, from analytic
properties and an independent restatement.

BSDFs (lambertian.h:10-29, microfacet.h:1-123, materials.h:7-43):
  * the pdf a sample reports equals the pdf evaluated at the sampled
    direction, and so does the BSDF value (Lambert exactly; Torrance-Sparrow
    within float rounding of the recomputed half vector raised to the Blinn
    exponent);
  * reciprocity, f(wo, wi) = f(wi, wo);
  * the pdf integrates to 1 over the sphere (midpoint quadrature);
  * directional albedo: Lambert gives its albedo, Torrance-Sparrow with the
    V-cavity G and a Fresnel term <= 1 stays at or below 1;
  * closed forms at normal incidence, with and without the reference's
    fixed IOR and exponent-is-roughness behaviours;
  * Kolmogorov-Smirnov tests of the cosine-hemisphere and Blinn half-vector
    sampling distributions.
Environment (image.cpp:68-389 as restated, lights.h:20-55,
envMapSample.h:23-123):
  * the marginal and conditional CDFs equal an independent float64 build
    from the image: FP16 texels, Rec.709 luminance, separable 3-tap
    Gaussian of sigma 0.75 px with clamp to edge, sin(theta) weight;
  * the pdf a sample reports equals the pdf evaluated along its direction;
  * a chi-square test of sampled directions against the texel
    probabilities of that independent build;
  * the pdf integrates to 1 over the sphere;
  * the background rotation turns the map about +Y, for evaluation and
    sampling alike.
"""
import numpy as np
import pytest

LAMBERT = (0, (0.8, 0.5, 0.3), 0.0)
METAL = (1, (0.9, 0.8, 0.5), 0.3)          # Blinn exponent 2 / 0.09 - 2 = 20.2
PLASTIC = (2, (0.2, 0.5, 0.9), 0.1)        # exponent 198, reflectance 1 (plastic.h:15,26)
SHINY = (1, (0.9, 0.9, 0.9), 0.05)         # exponent 798
WO = np.array([0.3, 0.8, 0.52]) / np.linalg.norm([0.3, 0.8, 0.52])


def upper_hemisphere(rng, n):
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:, 1] = np.abs(d[:, 1])
    return d


def sphere_grid(n_cos, n_phi):
    """Midpoints of an equal-area (cos theta, phi) grid and the cell solid angle."""
    ct = -1 + (np.arange(n_cos) + 0.5) * (2.0 / n_cos)
    ph = (np.arange(n_phi) + 0.5) * (2 * np.pi / n_phi)
    c, p = np.meshgrid(ct, ph, indexing="ij")
    s = np.sqrt(1 - c * c)
    return np.stack([s * np.cos(p), c, s * np.sin(p)], -1).reshape(-1, 3), (2.0 / n_cos) * (2 * np.pi / n_phi)


@pytest.mark.parametrize("mat", [LAMBERT, METAL, PLASTIC, SHINY], ids=["lambert", "metal", "plastic", "shiny"])
def test_bsdf_sample_agrees_with_eval_and_is_reciprocal(orc, mat):
    rng = np.random.default_rng(mat[0] * 10 + int(mat[2] * 100))
    n = 100000
    wo = upper_hemisphere(rng, n)
    wi, f, pdf = orc.bsdf_sample(mat, wo, rng.random((n, 2)))
    fe, pe = orc.bsdf_eval(mat, wo, wi)
    up = (wi[:, 1] > 1e-3) & (pdf > 0)
    assert up.mean() > 0.8
    rel_pdf = np.abs(pe[up] - pdf[up]) / pdf[up]
    rel_f = np.abs(fe[up] - f[up]).max(1) / np.abs(f[up]).max(1)
    fr, _ = orc.bsdf_eval(mat, wi[up], wo[up])
    rel_r = np.abs(fr - fe[up]).max(1) / np.abs(fe[up]).max(1)
    if mat[0] == 0:
        assert rel_pdf.max() == 0 and rel_f.max() == 0 and rel_r.max() == 0
        np.testing.assert_array_equal(pdf, (wi[:, 1] / np.float32(3.14159265359)).astype(np.float32))
    else:
        for rel in (rel_pdf, rel_f, rel_r):
            assert np.quantile(rel, 0.999) < 1e-3 and rel.max() < 2e-2


@pytest.mark.parametrize("mat,grid", [(LAMBERT, (500, 1000)), (METAL, (1000, 2000)), (PLASTIC, (2000, 4000))],
                         ids=["lambert", "metal", "plastic"])
def test_bsdf_pdf_integrates_to_one(orc, mat, grid):
    d, dw = sphere_grid(*grid)
    _, p = orc.bsdf_eval(mat, np.tile(WO, (len(d), 1)), d)
    if mat[0] == 0:
        p = np.where(d[:, 1] > 0, p, 0)          # the cosine pdf lives on the upper hemisphere
    assert abs(p.astype(np.float64).sum() * dw - 1.0) < 1e-5


@pytest.mark.parametrize("mat", [LAMBERT, METAL, PLASTIC, SHINY], ids=["lambert", "metal", "plastic", "shiny"])
def test_bsdf_directional_albedo(orc, mat):
    rng = np.random.default_rng(3)
    n = 200000
    wi, f, pdf = orc.bsdf_sample(mat, np.tile(WO, (n, 1)), rng.random((n, 2)))
    ok = (wi[:, 1] > 0) & (pdf > 0)
    w = np.where(ok[:, None], f.astype(np.float64) * wi[:, 1:2] / np.where(ok, pdf, 1)[:, None], 0.0)
    mean, err = w.mean(0), w.std(0) / np.sqrt(n)
    if mat[0] == 0:
        assert np.all(np.abs(mean - np.array(mat[1])) < 5 * err + 1e-3)
    else:
        assert np.all(mean <= 1 + 5 * err)
        assert np.all(mean > 0.3)


def independent_env_build(rgb):
    """Texel probabilities and CDFs of the environment, restated in float64."""
    t = np.clip(rgb, -65504, 65504).astype(np.float16).astype(np.float64)
    lum = t[..., 0] * 0.2126 + t[..., 1] * 0.7152 + t[..., 2] * 0.0722
    g = np.exp(-1 / (2 * 0.75 ** 2))
    k = np.array([g, 1.0, g]) / (1 + 2 * g)
    p = np.pad(lum, 1, mode="edge")
    bx = k[0] * p[:, :-2] + k[1] * p[:, 1:-1] + k[2] * p[:, 2:]
    blur = k[0] * bx[:-2] + k[1] * bx[1:-1] + k[2] * bx[2:]
    h, w = lum.shape
    func = np.maximum(blur, 0) * np.sin(np.pi * (np.arange(h) + 0.5) / h)[:, None]
    rows = func.sum(1)
    cdf_u = np.concatenate([np.zeros((h, 1)), np.cumsum(func, 1)], 1) / rows[:, None]
    cdf_v = np.concatenate([[0.0], np.cumsum(rows)]) / rows.sum()
    integral = rows.sum() / (w * h) * 2 * np.pi ** 2
    return func / func.sum(), cdf_u, cdf_v, integral


@pytest.fixture(scope="module")
def sky(orc):
    rng = np.random.default_rng(0)
    h, w = 32, 64
    rgb = rng.lognormal(0, 1.5, (h, w, 3)).astype(np.float32)
    rgb[5:8, 40:44] *= 50                        # a small bright sun
    return rgb, orc.Env(rgb)


def test_env_cdfs_match_independent_build(sky):
    rgb, env = sky
    _, cdf_u, cdf_v, integral = independent_env_build(rgb)
    assert np.abs(env.cdf_u - cdf_u).max() < 2e-7
    assert np.abs(env.cdf_v - cdf_v).max() < 2e-7
    assert abs(env.integral - integral) < 1e-6 * integral


def test_env_sample_pdf_and_radiance_agree_with_eval(orc, sky):
    _, env = sky
    rng = np.random.default_rng(1)
    d, L, pdf = orc.env_sample(env, rng.random((200000, 2)))
    Le, pe = orc.env_eval(env, d)
    assert np.quantile(np.abs(pe - pdf) / pdf, 0.999) < 1e-4 and (np.abs(pe - pdf) / pdf).max() < 1e-3
    assert (np.abs(Le - L).max(1) / np.abs(L).max(1)).max() < 1e-3


def test_env_sampler_chi_square(orc, sky):
    stats = pytest.importorskip("scipy.stats")
    rgb, env = sky
    p_tex, _, _, _ = independent_env_build(rgb)
    rng = np.random.default_rng(2)
    n = 400000
    d, _, _ = orc.env_sample(env, rng.random((n, 2)))
    u = ((np.arctan2(d[:, 2], d[:, 0]) + np.pi) / (2 * np.pi)) % 1.0
    v = np.arccos(np.clip(d[:, 1], -1, 1)) / np.pi
    bu, bv = 16, 8
    h, w = p_tex.shape
    iu = np.minimum((u * bu).astype(int), bu - 1)
    iv = np.minimum((v * bv).astype(int), bv - 1)
    obs = np.bincount(iv * bu + iu, minlength=bu * bv)
    exp = p_tex.reshape(bv, h // bv, bu, w // bu).sum((1, 3)).reshape(-1) * n
    chi = ((obs - exp) ** 2 / exp).sum()
    assert stats.chi2.sf(chi, bu * bv - 1) > 1e-3
    # and a plain bias check: the sun's bins hold their share
    sun = np.zeros((h, w), bool)
    sun[5:8, 40:44] = True
    share = ((np.floor(v * h).astype(int) >= 5) & (np.floor(v * h).astype(int) < 8) &
             (np.floor(u * w).astype(int) >= 40) & (np.floor(u * w).astype(int) < 44)).mean()
    assert abs(share - p_tex[sun].sum()) < 5 * np.sqrt(p_tex[sun].sum() / n)


def test_env_pdf_integrates_to_one(orc, sky):
    _, env = sky
    d, dw = sphere_grid(1000, 2000)
    _, p = orc.env_eval(env, d)
    assert abs(p.astype(np.float64).sum() * dw - 1.0) < 1e-3


@pytest.mark.parametrize("quirks", [0, "reference"])
def test_torrance_sparrow_at_normal_incidence(orc, quirks):
    """wo = wi = the normal gives wh = the normal, G = 1 and Schlick's F = F0,
    so f = R D(0) F0 / 4 and pdf = (e + 1) / (8 pi) (microfacet.h:19-37,
    64-91).  With the reference's quirks F0 comes from the fixed IOR 7.3
    ((6.3 / 8.3)^2), the Blinn exponent is the roughness field, and the
    metal's reflectance scales D; without them F0 is the material's colour,
    the exponent 2 / r^2 - 2 and D is unscaled."""
    from voxeltoy_gb300 import _lib as L
    q = 0 if quirks == 0 else (L.VT_QUIRK_FIXED_IOR | L.VT_QUIRK_EXPONENT_IS_ROUGHNESS)
    up = np.array([[0.0, 1.0, 0.0]])
    for t, albedo, rough in [(1, (0.9, 0.6, 0.3), 0.25), (1, (0.5, 0.5, 0.5), 0.5), (2, (0.2, 0.5, 0.9), 0.1)]:
        a = np.array(albedo, np.float32).astype(np.float16).astype(np.float64)   # FP16 palette records
        r = float(np.float16(rough))
        f, pdf = orc.bsdf_eval((t, albedo, rough), up, up, quirks=q)
        refl = a if t == 1 else np.ones(3)
        if q:
            e = r
            f0 = np.full(3, ((1 - 7.3) / (1 + 7.3)) ** 2)
            d_scale = refl
        else:
            e = max(2 / max(r * r, 1e-6) - 2, 0.0)
            f0 = refl
            d_scale = np.ones(3)
        want = d_scale * (e + 2) / (2 * np.pi) * f0 / 4
        np.testing.assert_allclose(f[0], want, rtol=2e-5)
        np.testing.assert_allclose(pdf[0], (e + 1) / (8 * np.pi), rtol=2e-5)


def test_env_rotation_turns_the_map_about_y(orc, sky):
    """uvCoordFromVector (coordinates.h:97-109) adds the rotation to the
    azimuth atan2(z, x): looking along d with rotation rho sees what d turned
    by rho about +Y sees without it; sampling with rho returns directions
    turned by -rho, with the same pdf."""
    _, env = sky
    rng = np.random.default_rng(5)
    d = rng.normal(size=(20000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for rho in (0.5, 2.0, -1.25):
        c, s = np.cos(rho), np.sin(rho)
        # azimuth phi = atan2(z, x) -> phi + rho
        turned = np.stack([c * d[:, 0] - s * d[:, 2], d[:, 1], s * d[:, 0] + c * d[:, 2]], 1)
        L1, p1 = orc.env_eval(env, d, rotation=rho)
        L0, p0 = orc.env_eval(env, turned)
        assert np.quantile(np.abs(L1 - L0).max(1) / np.abs(L0).max(1), 0.99) < 1e-3
        u = rng.random((5000, 2))
        ds, _, ps = orc.env_sample(env, u, rotation=rho)
        d0, _, p00 = orc.env_sample(env, u)
        back = np.stack([c * ds[:, 0] - s * ds[:, 2], ds[:, 1], s * ds[:, 0] + c * ds[:, 2]], 1)
        assert np.abs(back - d0).max() < 1e-4
        np.testing.assert_array_equal(ps, p00)


def test_sampled_directions_follow_their_distributions(orc):
    """Kolmogorov-Smirnov tests of the samplers' published distributions:
    the cosine-weighted hemisphere of sampling.h:2-20 has P(cos theta <= t)
    = t^2; the Blinn half vector of sampleD (microfacet.h:41-61), cos theta_h
    = u^(1 / (e + 1)), has P(cos theta_h <= t) = t^(e + 1)."""
    stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(6)
    n = 100000
    wo = np.tile(WO, (n, 1))
    wi, _, _ = orc.bsdf_sample(LAMBERT, wo, rng.random((n, 2)))
    assert stats.kstest(wi[:, 1].astype(np.float64), lambda t: np.clip(t, 0, 1) ** 2).pvalue > 1e-3
    for mat, e in ((METAL, 2 / np.float16(0.3) ** 2 - 2), (PLASTIC, 2 / np.float16(0.1) ** 2 - 2)):
        wi, _, _ = orc.bsdf_sample(mat, wo, rng.random((n, 2)))
        wh = wi.astype(np.float64) + wo
        wh /= np.linalg.norm(wh, axis=1, keepdims=True)
        assert stats.kstest(wh[:, 1], lambda t: np.clip(t, 0, 1) ** (float(e) + 1)).pvalue > 1e-3
