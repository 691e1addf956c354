"""The oracle built with AddressSanitizer and UndefinedBehaviorSanitizer
(errors abort) renders small cases of every configuration family, with
every reference quirk and the noise-table walk, and voxelizes a mesh:
out-of-bounds accesses, use-after-free and undefined arithmetic (signed
overflow, bad shifts, misaligned loads) in the restatement stop the run.
The sanitized library runs in a child process with libasan preloaded."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import numpy as np
import sys
sys.path.insert(0, 'tests')
from oracle import binding as orc
from voxeltoy_gb300 import scenes as S
from helpers import reference_config
cfgs = [S.config1(edge=24, width=20, height=16, make=orc), S.config2(edge=20, width=16, height=14,
        env_size=(32, 16), make=orc)]
for cfg in cfgs:
    em = orc.emissive_list(cfg.voxels, cfg.palette) if cfg.env_rgb is not None else None
    sc = orc.Scene(cfg.voxels, cfg.palette, em)
    env = orc.Env(cfg.env_rgb) if cfg.env_rgb is not None else orc.Env()
    for prec in (32, 64):
        img, cnt = orc.render_average(cfg.camera, cfg.settings, sc, env, cfg.width, cfg.height, 3, prec, threads=2)
        assert np.isfinite(img).all() and cnt[0] == 3 * cfg.width * cfg.height
cfg = reference_config(edge=16, w=12, h=10)
sc = orc.Scene(cfg.voxels, cfg.palette, None)
img, cnt = orc.render_average(cfg.camera, cfg.settings, sc, orc.Env(), cfg.width, cfg.height, 2, 32, threads=2,
                              noise=orc.noise_table())
assert cnt[0] == 2 * cfg.width * cfg.height
v, f = S.fbm_displaced_icosphere(level=2)
g = orc.voxelize(v, f, (24, 20, 28), 1, placement=1)
assert g.sum() > 0
assert "libvt_oracle_asan" in open("/proc/self/maps").read()
print("SANITIZED_OK")
"""


def test_oracle_under_asan_and_ubsan():
    from oracle import build as ob
    ob.build(sanitize=True)
    asan = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    env = dict(os.environ, VT_ORACLE_SANITIZED="1", LD_PRELOAD=asan,
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=1", UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "SANITIZED_OK" in r.stdout, (r.stdout[-3000:], r.stderr[-6000:])
