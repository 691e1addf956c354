"""Accuracy of the single-precision GLSL builtins shared by the kernels and
the oracle's float build (sin, cos, pow, acos, atan2, log2, exp2, half
conversion), checked against float64 libm."""
import numpy as np
import pytest


def ulp_err(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    spacing = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    return np.abs(got - want) / spacing


def test_sin_cos(orc):
    x = np.linspace(-40.0, 40.0, 400001, dtype=np.float32)
    for fn, ref in ((0, np.sin), (1, np.cos)):
        got = orc.builtins(fn, x)
        want = ref(x.astype(np.float64))
        err = np.abs(got - want)
        # absolute error within 2 ulp of 1 (results near zero are checked absolutely)
        assert err.max() <= 2 * np.spacing(np.float32(1.0)), fn
        big = np.abs(want) > 0.1
        assert ulp_err(got[big], want[big]).max() <= 4


def test_pow(orc):
    rng = np.random.default_rng(0)
    x = rng.uniform(1e-6, 1.0, 200000).astype(np.float32)
    y = np.exp(rng.uniform(np.log(0.05), np.log(2000.0), x.size)).astype(np.float32)
    got = orc.builtins(2, x, y).astype(np.float64)
    want = np.power(x.astype(np.float64), y.astype(np.float64))
    ok = want > 1e-30
    rel = np.abs(got[ok] - want[ok]) / want[ok]
    # the error grows with |y log2 x| (one float rounding of the exponent)
    bound = 4e-7 * (1.0 + np.abs(y[ok] * np.log2(x[ok])))
    assert np.all(rel <= bound)
    # gamma of the tonemapper and Schlick's fifth power
    g = orc.builtins(2, np.float32([0.0, 1.0, 2.0, 1e-3]), np.float32([1 / 2.2] * 4))
    np.testing.assert_allclose(g, np.power([0.0, 1.0, 2.0, 1e-3], 1 / 2.2), rtol=1e-6)
    # the fifth power is three products, within 3 ulp
    x5 = rng.uniform(1e-3, 1.0, 10000).astype(np.float32)
    got5 = orc.builtins(2, x5, np.full_like(x5, 5.0)).astype(np.float64)
    want5 = x5.astype(np.float64) ** 5
    assert np.all(np.abs(got5 - want5) <= 3 * np.spacing(want5.astype(np.float32)).astype(np.float64))
    # conventions where GLSL leaves pow undefined
    assert orc.builtins(2, np.float32([-0.5, 0.0, -2.0]), np.float32([5.0, 3.0, 0.0])).tolist() == [0.0, 0.0, 1.0]


def test_acos_atan2(orc):
    x = np.linspace(-1.0, 1.0, 200001, dtype=np.float32)
    got = orc.builtins(3, x)
    assert np.abs(got - np.arccos(x.astype(np.float64))).max() < 4e-7
    assert orc.builtins(3, np.float32([1.5, -1.5])).tolist() == [0.0, np.float32(np.pi)]
    rng = np.random.default_rng(1)
    y = rng.normal(size=200000).astype(np.float32)
    xx = rng.normal(size=200000).astype(np.float32)
    got = orc.builtins(4, y, xx)
    assert np.abs(got - np.arctan2(y.astype(np.float64), xx.astype(np.float64))).max() < 8e-7
    assert orc.builtins(4, np.float32([0.0]), np.float32([0.0])).tolist() == [0.0]


def test_log2_exp2(orc):
    x = np.exp(np.linspace(-80, 80, 100001)).astype(np.float32)
    got = orc.builtins(5, x)
    want = np.log2(x.astype(np.float64))
    tol = np.maximum(2 * np.spacing(np.abs(want).astype(np.float32)), 3e-7)
    assert np.all(np.abs(got - want) <= tol)
    y = np.linspace(-140, 120, 100001).astype(np.float32)
    got = orc.builtins(6, y).astype(np.float64)
    want = np.exp2(y.astype(np.float64))
    ok = want > 1.2e-38
    assert (np.abs(got[ok] - want[ok]) / want[ok]).max() < 3e-7


def test_half_conversion_matches_ieee(orc):
    rng = np.random.default_rng(2)
    x = np.concatenate([
        rng.normal(0, 1, 50000), rng.normal(0, 1e4, 50000), rng.uniform(-7e-5, 7e-5, 50000),
        [0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e9, -1e9, 6.0e-8, 2.98e-8, 5.96e-8, 1e-10],
    ]).astype(np.float32)
    got = orc.builtins(7, x)
    want = x.astype(np.float16).astype(np.float32)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
