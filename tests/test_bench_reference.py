"""The reference arm of bench.py runs the oracle alone.

Its inputs are built by the numpy generators and the oracle's own camera and
settings helpers; the CUDA library must not be mapped into that process.
The helpers must give the same camera and settings as the library's
vt_camera_orbit / vt_settings_default (host code, no GPU needed).
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_maps_no_product_library():
    code = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'config1', '--steps', '1', '--warmup', '0',"
        " '--cpu-seconds', '0.3']\n"
        "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit:\n    pass\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPPED', 'libvoxeltoy' in maps, 'vt_oracle' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert lines[-1] == "MAPPED False True", lines[-1]


def test_oracle_camera_and_settings_match_the_library():
    from oracle import binding as orc
    from voxeltoy_gb300 import scenes as S
    from voxeltoy_gb300 import _lib as L
    for args in [dict(), dict(theta_deg=33.0, phi_deg=-71.5, distance=1234.5, lens=L.VT_LENS_THIN_LENS,
                                aperture=20.0), dict(lens=L.VT_LENS_ORTHOGRAPHIC, fov_deg=30.0, focus=77.0)]:
        a, b = S.orbit_camera(**args), orc.orbit_camera(**args)
        for name, _t in orc.OrcCamera._fields_:
            va, vb = getattr(a, name), getattr(b, name)
            va = np.array(list(va) if hasattr(va, "__len__") else [va], np.float32)
            vb = np.array(list(vb) if hasattr(vb, "__len__") else [vb], np.float32)
            assert np.array_equal(va.view(np.uint32), vb.view(np.uint32)), name
    for kw in [dict(max_bounces=8, rr_start=3, seed=2), dict(max_bounces=4)]:
        a, b = S.physical_settings(**kw), orc.physical_settings(**kw)
        for name, _t in L.RenderSettings._fields_:
            va, vb = getattr(a, name), getattr(b, name)
            assert (list(va) if hasattr(va, "__len__") else va) == (list(vb) if hasattr(vb, "__len__") else vb), name
    # bitwise equality of the defaults too
    d = L.RenderSettings()
    L.call("vt_settings_default", C.byref(d))
    o = orc.OrcSettings()
    orc.lib().orc_settings_default(C.byref(o))
    assert bytes(d) == bytes(o)[:C.sizeof(d)]
