"""The committed golden fixtures of tests/golden (written by
tests/golden/make_golden.py).

oracle_frames.npz holds small frames of the CPU oracle with all of their
inputs.  On the CPU the oracle must still reproduce them bit for bit (a
change of the checker shows up here first); on the GPU the CUDA path must
reproduce them through the C ABI without the oracle in the loop."""
import ctypes as C
import os

import numpy as np
import pytest

from voxeltoy_gb300 import _lib as L

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("config1", "config2", "reference")


@pytest.fixture(scope="module")
def frames():
    with np.load(os.path.join(HERE, "oracle_frames.npz")) as d:
        return {k: d[k] for k in d.files}


def inputs(frames, name):
    pal = [(int(r[0]), tuple(float(x) for x in r[1:4]), tuple(float(x) for x in r[4:7]), float(r[7]))
           for r in frames[f"{name}/palette"]]
    cam = L.Camera.from_buffer_copy(frames[f"{name}/camera"].tobytes())
    st = L.RenderSettings.from_buffer_copy(frames[f"{name}/settings"].tobytes())
    env = frames[f"{name}/env"]
    w, h = (int(v) for v in frames[f"{name}/size"])
    return frames[f"{name}/voxels"], pal, frames[f"{name}/emissive"], (env if env.size else None), cam, st, w, h


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden_frames(orc, frames, name):
    vox, pal, em, env, cam, st, w, h = inputs(frames, name)
    osc = orc.Scene(vox, pal, em if len(em) else None)
    oenv = orc.Env(env) if env is not None else orc.Env()
    noise = orc.noise_table() if st.rng_mode == L.VT_RNG_NOISE_TABLE else None
    for smp in frames[f"{name}/samples"]:
        rgba, hits, _ = orc.render_samples(cam, st, osc, oenv, w, h, int(smp), 32, noise=noise)
        np.testing.assert_array_equal(hits, frames[f"{name}/hits{smp}"])
        np.testing.assert_array_equal(rgba.view(np.uint32), frames[f"{name}/rgba{smp}"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_reproduces_golden_frames(ctx, frames, name):
    from helpers import close_all
    from voxeltoy_gb300 import Env, Job, Scene
    vox, pal, em, env, cam, st, w, h = inputs(frames, name)
    sc = Scene.dense(ctx, vox, pal, emissive=em if len(em) else None)
    ev = Env(ctx, env) if env is not None else None
    job = Job(ctx, sc, ev, cam, st, w, h)
    try:
        np.testing.assert_array_equal(sc.emissive(), em)
        for smp in frames[f"{name}/samples"]:
            rgba, hits, _ = job.samples_diag(int(smp))
            np.testing.assert_array_equal(hits, frames[f"{name}/hits{smp}"])
            np.testing.assert_array_equal(rgba.view(np.uint32), frames[f"{name}/rgba{smp}"])
    finally:
        close_all(job, ev, sc)
