"""vt_cli: the C++ host program (voxeltoy_gb300/host/vt_cli.cpp) that drives
the renderer through the C ABI alone.

On the CPU: it is built, prints its usage, and fails loudly (status 1 and
the library's message) when there is no GPU.  On the GPU: it reproduces the
golden oracle frames bit for bit, and its .vox render equals the same render
through the Python binding."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from voxeltoy_gb300 import _lib as L
from voxeltoy_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def cli():
    B.build()
    assert B.CLI.exists()
    return str(B.CLI)


def write_frame_dir(d, frames, name, sample):
    vox = frames[f"{name}/voxels"]
    rz, ry, rx = vox.shape
    w, h = (int(v) for v in frames[f"{name}/size"])
    pal = frames[f"{name}/palette"].astype(np.float32)
    em = frames[f"{name}/emissive"].astype(np.int32)
    env = frames[f"{name}/env"].astype(np.float32)
    eh, ew = env.shape[:2] if env.size else (0, 0)
    with open(os.path.join(d, "meta.txt"), "w") as f:
        f.write(f"{rx} {ry} {rz} {w} {h} {sample} {len(pal)} {len(em)} {ew} {eh}\n")
    vox.astype(np.uint8).tofile(os.path.join(d, "voxels.u8"))
    pal.tofile(os.path.join(d, "palette.f32"))
    em.tofile(os.path.join(d, "emissive.i32"))
    if env.size:
        env.tofile(os.path.join(d, "env.f32"))
    frames[f"{name}/camera"].tofile(os.path.join(d, "camera.bin"))
    frames[f"{name}/settings"].tofile(os.path.join(d, "settings.bin"))
    return w, h


def load_frames():
    with np.load(os.path.join(HERE, "golden", "oracle_frames.npz")) as z:
        return {k: z[k] for k in z.files}


def test_cli_usage_and_missing_inputs(cli, tmp_path):
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([cli, "frame", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 2


def test_cli_fails_loudly_without_a_device(cli, tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    write_frame_dir(str(tmp_path), load_frames(), "config1", 0)
    r = subprocess.run([cli, "frame", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "vt_create" in r.stderr
    assert not (tmp_path / "rgba.f32").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["config1", "config2", "reference"])
def test_cli_reproduces_golden_frames(cli, tmp_path, name):
    frames = load_frames()
    sample = int(frames[f"{name}/samples"][0])
    w, h = write_frame_dir(str(tmp_path), frames, name, sample)
    r = subprocess.run([cli, "frame", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rgba = np.fromfile(tmp_path / "rgba.f32", np.uint32).reshape(h, w, 4)
    hits = np.fromfile(tmp_path / "hits.i32", np.int32).reshape(h, w, 4)
    np.testing.assert_array_equal(hits, frames[f"{name}/hits{sample}"])
    np.testing.assert_array_equal(rgba, frames[f"{name}/rgba{sample}"])


@pytest.mark.gpu
def test_cli_vox_render_equals_binding(cli, ctx, tmp_path):
    from helpers import close_all
    from test_formats import vox_file
    from voxeltoy_gb300 import Job, Scene, default_settings
    from voxeltoy_gb300 import formats as F
    rng = np.random.default_rng(5)
    size = (24, 20, 16)
    pts = {tuple(int(rng.integers(0, s)) for s in size) for _ in range(1500)}
    data = vox_file(size, [(x, y, z, int(rng.choice([3, 17, 40]))) for x, y, z in sorted(pts)])
    (tmp_path / "in.vox").write_bytes(data)
    w, h, spp = 40, 32, 4
    r = subprocess.run([cli, "vox", str(tmp_path / "in.vox"), str(tmp_path / "out.pfm"), str(w), str(h), str(spp)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Mpaths/s" in r.stdout
    got = F.image_decode((tmp_path / "out.pfm").read_bytes())
    sc = Scene.from_vox(ctx, data, L.VT_SCENE_PRUNE_EMISSIVE)
    job = None
    try:
        info = sc.info()
        cam = L.Camera()
        L.call("vt_camera_default", C.byref(cam))
        lo = (C.c_float * 3)(*info.bounds_min)
        hi = (C.c_float * 3)(*info.bounds_max)
        L.call("vt_camera_focus_on_bounds", C.byref(cam), lo, hi)
        st = default_settings()
        st.max_samples = spp
        job = Job(ctx, sc, None, cam, st, w, h)
        job.render(spp)
        want = job.readback()[::-1, :, :3]
        np.testing.assert_array_equal(got.view(np.uint32), np.ascontiguousarray(want).view(np.uint32))
    finally:
        close_all(job, sc)
