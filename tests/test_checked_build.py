"""The bounds-checked build (libvoxeltoy_checked.so, VT_CHECKED): in a child
process that loads it, the golden frames (per-sample radiance and first
hits of the config-1, config-2 and all-quirks cases) come out bit for bit as
in the fixtures, accumulated wavefront and plain frames equal the release
build's, and no gather of the path tracer fell outside its buffer (the
check word stays 0).  The checks record and skip; nothing traps."""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu

FRAMES = r"""
import ctypes as C, hashlib, json, sys
import numpy as np
sys.path.insert(0, 'tests')
from voxeltoy_gb300 import Context, Env, Job, Scene
from voxeltoy_gb300 import _lib as L
from helpers import small_config1, small_config2, reference_config, close_all
out = {}
ctx = Context(0)
for name, cfg in [("config1", small_config1(edge=40, w=48, h=40)), ("config2", small_config2(edge=36, w=40, h=36)),
                  ("reference", reference_config(edge=32, w=32, h=28))]:
    cfg.settings.max_samples = 1 << 20
    sc = Scene.dense(ctx, cfg.voxels, cfg.palette, flags=cfg.scene_flags)
    ev = Env(ctx, cfg.env_rgb) if cfg.env_rgb is not None else None
    for kernel in (1, 2):
        ctx.set_kernel(kernel)
        job = Job(ctx, sc, ev, cfg.camera, cfg.settings, cfg.width, cfg.height)
        job.render(6)
        out[f"{name}/{kernel}"] = hashlib.blake2b(job.readback().tobytes(), digest_size=16).hexdigest()
        job.close()
    close_all(ev, sc)
w, en = C.c_uint32(), C.c_int32()
L.call("vt_diag_check_word", ctx.h, C.byref(w), C.byref(en))
out["check_word"], out["checked"] = w.value, en.value
out["library"] = [l.split()[-1] for l in open("/proc/self/maps") if "libvoxeltoy" in l][0]
ctx.close()
print("RESULT " + json.dumps(out))
"""

GOLDEN = r"""
import sys
sys.path.insert(0, 'tests')
import pytest
sys.exit(pytest.main(['-q', '-x', '-m', 'gpu', '-p', 'no:cacheprovider', 'tests/test_golden.py']))
"""


def run_child(code, checked):
    env = dict(os.environ)
    env.pop("VOXELTOY_CHECKED", None)
    if checked:
        env["VOXELTOY_CHECKED"] = "1"
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    return r.stdout


def test_checked_build_renders_like_the_release_build():
    from voxeltoy_gb300 import build as B
    B.build(checked=True)
    rel = json.loads(run_child(FRAMES, False).split("RESULT ", 1)[1])
    chk = json.loads(run_child(FRAMES, True).split("RESULT ", 1)[1])
    assert rel["checked"] == 0 and rel["library"].endswith("libvoxeltoy.so")
    assert chk["checked"] == 1 and chk["library"].endswith("libvoxeltoy_checked.so")
    assert chk["check_word"] == 0
    for k in rel:
        if "/" in k:
            assert chk[k] == rel[k], k


def test_checked_build_reproduces_the_golden_frames():
    from voxeltoy_gb300 import build as B
    B.build(checked=True)
    out = run_child(GOLDEN, True)
    assert "passed" in out and "failed" not in out
