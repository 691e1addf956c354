"""Known-answer checks of the CPU oracle.

Pins the oracle on the only golden vectors the reference itself documents
(the CDF worked example of src/renderer/image.cpp:107-154 and the binary
search example of src/shaders/envLight/envMapSample.h:10-21), on the
published Philox-4x32-10 known-answer vectors, and on analytic answers.
"""
import json
import os

import numpy as np
import pytest

# the examples as tests/golden/reference_examples.json holds them
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_examples.json")) as _f:
    GOLDEN = json.load(_f)
# image.cpp:107-124 -- one row of intensities and its normalised CDF
ROW0 = GOLDEN["cdf_rows"]["rows"][0]
ROW0_CDF = GOLDEN["cdf_rows"]["row0_cdf"]
# image.cpp:144-154 -- second row (sum 12) and a last row taking the total to 150
ROW1 = GOLDEN["cdf_rows"]["rows"][1]
LAST = GOLDEN["cdf_rows"]["rows"][2]


def test_cdf_row_example_reference_float(orc):
    cu, cv = orc.cdf_reference_float(np.array([ROW0], np.float32))
    np.testing.assert_allclose(cu[0], ROW0_CDF, rtol=0, atol=1e-7)
    assert cv.tolist() == [0.0, 1.0]


@pytest.mark.parametrize("chunk", [0, 32, 2])
def test_cdf_row_example_fp64(orc, chunk):
    cu, cv, _ = orc.cdf_from_function(np.array([ROW0], np.float32), chunk=chunk)
    assert cu[0].tolist() == [np.float32(x) for x in ROW0_CDF]


def test_cdf_marginal_example(orc):
    func = np.array([ROW0, ROW1, LAST], np.float32)
    _, cv, _ = orc.cdf_from_function(func)
    np.testing.assert_array_equal(cv, np.float32([0.0, 10 / 150, 22 / 150, 1.0]))
    assert f"{cv[1]:.2f}"[:3] == "0.0" and int(cv[1] * 100) == 6      # the comment's 0.06
    assert int(cv[2] * 100) == 14                                       # the comment's 0.14
    _, cvr = orc.cdf_reference_float(func)
    np.testing.assert_allclose(cvr, cv, rtol=0, atol=2e-7)


def test_cdf_black_rows_are_uniform(orc):
    func = np.zeros((3, 4), np.float32)
    func[1] = [0, 3, 0, 1]
    cu, cv, integral = orc.cdf_from_function(func)
    assert cu[0].tolist() == [0.0, 0.25, 0.5, 0.75, 1.0]
    assert cu[1].tolist() == [0.0, 0.0, 0.75, 0.75, 1.0]
    assert cv.tolist() == [0.0, 0.0, 1.0, 1.0]
    allblack, cvb, ib = orc.cdf_from_function(np.zeros((2, 2), np.float32))
    assert cvb.tolist() == [0.0, 0.5, 1.0] and ib == 0.0


def test_binary_search_example(orc):
    # envMapSample.h:10-21: u = 0.7 lands in the bracket starting at index 3
    ex = GOLDEN["binary_search"]
    assert ex["queries"][0] == [0.7, 3]
    for u, k in ex["queries"]:
        assert orc.binary_search(ex["cdf"], u) == k


def test_philox_known_answers(orc):
    # Philox-4x32-10 known-answer vectors published with the algorithm (Salmon et al. 2011)
    for c in GOLDEN["philox4x32_10"]["cases"]:
        assert orc.philox(c["ctr"], c["key"]).tolist() == c["out"]


def test_constant_env_integral(orc):
    # a constant image L gives uniform CDFs and integral 2 pi^2 * L * mean(sin theta)
    w, h = 16, 8
    rgb = np.full((h, w, 3), 2.0, np.float32)
    env = orc.Env(rgb, chunk=0)
    np.testing.assert_allclose(env.cdf_u[0], np.arange(w + 1) / w, atol=1e-7)
    st = np.sin(np.pi * (np.arange(h) + 0.5) / h)
    np.testing.assert_allclose(env.cdf_v, np.concatenate([[0], np.cumsum(st) / st.sum()]), atol=2e-7)
    lum = 2.0 * (0.2126 + 0.7152 + 0.0722)
    assert env.integral == pytest.approx(2 * np.pi ** 2 * lum * st.mean(), rel=1e-6)


def test_delta_env_step_cdf(orc):
    w, h = 32, 16
    rgb = np.zeros((h, w, 3), np.float32)
    rgb[5, 9] = 100.0
    env = orc.Env(rgb, chunk=32)
    # after the 3x3 blur only rows 4..6 carry weight and row 5's mass sits in columns 8..10
    cv = env.cdf_v
    assert cv[4] == 0.0 and cv[7] == 1.0
    assert env.cdf_u[5][8] == 0.0 and env.cdf_u[5][11] == 1.0


def test_prune_emissive_against_numpy(orc):
    rng = np.random.default_rng(5)
    g = (rng.random((12, 10, 9)) < 0.6).astype(np.uint8)
    g[3:8, 3:8, 3:8] = 1
    em = np.flatnonzero(g.ravel()).astype(np.int32)
    rng.shuffle(em)
    pruned = orc.prune_emissive(g, em)

    def visible(i):
        z, rem = divmod(int(i), 10 * 9)
        y, x = divmod(rem, 9)
        for dx, dy, dz in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]:
            nx, ny, nz = x + dx, y + dy, z + dz
            if not (0 <= nx < 9 and 0 <= ny < 10 and 0 <= nz < 12) or g[nz, ny, nx] == 0:
                return True
        return False

    keep = [v for v in em if visible(v)]
    assert sorted(pruned.tolist()) == sorted(keep)
    # swap-with-last removal order (import.cpp:180-203)
    lst = em.tolist()
    i = 0
    while i < len(lst):
        if not visible(lst[i]):
            lst[i] = lst[-1]
            lst.pop()
        else:
            i += 1
    assert pruned.tolist() == lst


def test_edit_mode_known_answers(orc):
    """editMode.fs on volumes with known answers: an empty volume shows the
    background (the path tracer's miss), and a full volume seen from above
    through its top faces shows them white and unshadowed (sqrt(-d.n) of a
    view from above; the shadow ray leaves upwards, so nothing halves it)."""
    from voxeltoy_gb300 import scenes as S
    cfg = S.config1(edge=8, width=12, height=10, spp=1)
    empty = np.zeros((8, 8, 8), np.uint8)
    osc, env = orc.Scene(empty, cfg.palette, None), orc.Env()
    a, ha, _ = orc.render_samples(cfg.camera, cfg.settings, osc, env, 12, 10, 0, integrator=1)
    b, hb, _ = orc.render_samples(cfg.camera, cfg.settings, osc, env, 12, 10, 0, integrator=0)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (ha[..., 3] == 0).all()
    full = np.ones((8, 8, 8), np.uint8)
    cam = S.orbit_camera(distance=2000.0, theta_deg=160.0, phi_deg=30.0)   # eye above the volume
    img, hits, _ = orc.render_samples(cam, cfg.settings, orc.Scene(full, cfg.palette, None), env, 12, 10, 0,
                                      integrator=1)
    top = (hits[..., 3] & 0x3f) == (1 | (2 << 2) | (1 << 4))       # normal (0, +1, 0)
    assert top.any()
    v = img[top][:, :3]
    assert np.all(v[:, 0] == v[:, 1]) and np.all(v[:, 1] == v[:, 2])   # white voxels
    assert np.all((v > 0.5) & (v <= 1.0))        # sqrt(cos) of a view from above, never halved by a shadow



def _wang_hash(seed):
    """Thomas Wang's 32-bit integer hash as random.h:3-11 writes it, in signed
    32-bit arithmetic (arithmetic right shifts, wrapping products)."""
    s = np.asarray(seed, np.int64).astype(np.int32)
    with np.errstate(over="ignore"):
        s = (s ^ np.int32(61)) ^ (s >> 16)
        s = (s.astype(np.int64) * 9).astype(np.uint32).astype(np.int32)
        s = s ^ (s >> 4)
        s = (s.astype(np.int64) * 0x27D4EB2D).astype(np.uint32).astype(np.int32)
        s = s ^ (s >> 15)
    return s


def test_noise_table_walk_against_restatement(orc):
    """randomNumberGeneratorOffset (random.h:13-18): offset = hash(x + 1024 y)
    ^ hash(sample), read as unsigned, split into (offset % 1024, offset / 1024
    % 1024); rand (:20-27) returns that texel and advances x, wrapping into
    the next row and from the last row to the first."""
    table = orc.noise_table()
    rng = np.random.default_rng(4)
    cases = [(int(x), int(y), int(s)) for x, y, s in zip(rng.integers(0, 4096, 40), rng.integers(0, 4096, 40),
                                                      rng.integers(0, 1 << 20, 40))]
    # a stream that starts at the end of a row: find one by search
    for s in range(200000):
        off = int((_wang_hash(0) ^ _wang_hash(s)).astype(np.uint32))
        if off % 1024 >= 1022:
            cases.append((0, 0, s))
            break
    wrapped = False
    for x, y, s in cases:
        off = int((_wang_hash(x + 1024 * y) ^ _wang_hash(s)).astype(np.uint32))
        ox, oy = off % 1024, (off // 1024) % 1024
        want = []
        for _ in range(4):
            want.append(table[oy, ox])
            ox = (ox + 1) % 1024
            if ox == 0:
                oy = (oy + 1) % 1024
                wrapped = True
        np.testing.assert_array_equal(orc.noise_walk(table, x, y, s, 4), np.array(want))
    assert wrapped


def test_wang_hash_restatement_is_the_published_function():
    """The restatement above against the hash written with plain Python
    integers modulo 2^32 (logical shifts of the two's-complement pattern
    differ from arithmetic ones only in the high bits that the sign fills)."""
    def ref(seed):
        m = 0xFFFFFFFF
        def sar(v, k):   # arithmetic shift of a 32-bit pattern
            v &= m
            return ((v >> k) | (m << (32 - k) & m if v & 0x80000000 else 0)) & m
        s = seed & m
        s = (s ^ 61) ^ sar(s, 16)
        s = (s * 9) & m
        s = s ^ sar(s, 4)
        s = (s * 0x27D4EB2D) & m
        s = s ^ sar(s, 15)
        return s
    for seed in [0, 1, 61, 1024, 123456789, 2 ** 31 - 1, -1, -2 ** 31, 987654]:
        assert int(_wang_hash(seed).astype(np.uint32)) == ref(seed)


def test_reference_cdf_size_and_box_shrink(orc):
    """The oracle's reference-size environment build: the shrunk size by the
    reference's float arithmetic (image.cpp:314-317), and the CDFs of the
    area-weighted box average of the FP16 texels, restated here in numpy."""
    for (w, h) in [(1024, 512), (777, 333), (300, 900), (512, 256), (4000, 3)]:
        m = np.float32(max(w, h))
        want = (w, h) if max(w, h) <= 512 else \
            (int(np.uint32(np.float32(w) / m * np.float32(512))), int(np.uint32(np.float32(h) / m * np.float32(512))))
        assert orc.cdf_size(w, h) == want, (w, h)
    w, h = 777, 333
    rgb = np.random.default_rng(4).random((h, w, 3)).astype(np.float32) * 5
    env = orc.Env(rgb, chunk=32, flags=1)
    cw, ch = orc.cdf_size(w, h)
    assert env.cdf_u.shape == (ch, cw + 1) and env.cdf_v.shape == (ch + 1,)
    half = rgb.astype(np.float16).astype(np.float64)
    sx, sy = w / cw, h / ch

    def weights(n_out, scale, n_in):
        m = np.zeros((n_out, n_in))
        for o in range(n_out):
            a, b = o * scale, (o + 1) * scale
            for i in range(int(np.floor(a)), min(int(np.ceil(b)), n_in)):
                m[o, i] = min(b, i + 1) - max(a, i)
        return m
    wx, wy = weights(cw, sx, w), weights(ch, sy, h)
    rows_avg = (wy @ half.reshape(h, w * 3)).reshape(ch, w, 3)                 # rows, then columns
    avg = np.einsum("yic,xi->yxc", rows_avg, wx, optimize=True) / (sx * sy)
    lum = (avg[..., 0].astype(np.float32) * np.float32(0.2126) + avg[..., 1].astype(np.float32) * np.float32(0.7152)) \
        + avg[..., 2].astype(np.float32) * np.float32(0.0722)
    got_cu, got_cv = env.cdf_u, env.cdf_v
    assert np.all(np.diff(got_cu, axis=1) >= 0) and got_cu[:, -1].max() == 1.0 and got_cv[-1] == 1.0
    # the shrunk luminance drives the marginal: compare against a direct float64 build of the CDF of lum
    ws, wm = 0.225610111284051620, 0.548779777431896800
    lp = np.pad(lum.astype(np.float64), 1, mode="edge")
    bl = ws * lp[1:-1, :-2] + wm * lp[1:-1, 1:-1] + ws * lp[1:-1, 2:]
    bp = np.pad(bl, ((1, 1), (0, 0)), mode="edge")
    bl = ws * bp[:-2] + wm * bp[1:-1] + ws * bp[2:]
    st = np.sin(np.pi * (np.arange(ch) + 0.5) / ch)
    func = np.maximum(bl, 0) * st[:, None]
    rows = func.sum(1)
    marg = np.concatenate([[0], np.cumsum(rows)]) / rows.sum()
    assert np.allclose(got_cv, marg, atol=2e-6)
