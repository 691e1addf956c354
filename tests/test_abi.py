"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; calls that need a device fail cleanly."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        names |= set(re.findall(r"VT_API\s+[\w\s\*]+?\b(vt_\w+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(vtlib):
    names = declared_functions()
    assert len(names) > 50
    missing = [n for n in sorted(names) if not hasattr(vtlib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    from voxeltoy_gb300 import _lib
    names = declared_functions() - {"vt_last_error"}
    assert names <= set(_lib.SIGNATURES), sorted(names - set(_lib.SIGNATURES))


def test_errors_without_device(vtlib):
    from voxeltoy_gb300 import _lib as L
    h = C.c_void_p()
    rc = vtlib.vt_scene_create(None, 4, 4, 4, None, None, 1, None, 0, 0, C.byref(h))
    assert rc == L.VT_EINVAL
    assert b"null" in vtlib.vt_last_error()
    s = L.RenderSettings()
    assert vtlib.vt_settings_default(C.byref(s)) == 0
    assert s.max_bounces == 1 and s.max_samples == 2048 * 2048 and abs(s.gamma - 2.2) < 1e-6
    assert s.quirks == L.VT_QUIRKS_REFERENCE and s.nee_emission_scale == 10.0


def test_no_oracle_in_product():
    """The product sources never reference the oracle."""
    for p in list((ROOT / "voxeltoy_gb300").rglob("*.py")) + list((ROOT / "voxeltoy_gb300" / "csrc").glob("*")):
        if p.is_file():
            text = p.read_text(errors="ignore")
            assert "oracle" not in text.lower() or p.name == "__init__.py" and "oracle" not in text, p
