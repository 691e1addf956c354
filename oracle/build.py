"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/vt_oracle.cpp with g++ into oracle/_build/libvt_oracle.so.
Contraction of multiply-adds is disabled (-ffp-contract=off) so that the
single-precision build evaluates the same IEEE operations as the GPU kernels.
No architecture-specific flags: the same source gives the same results on
x86_64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "vt_oracle.cpp"
HDRS = [HERE / "vt_oracle.h", HERE.parent / "voxeltoy_gb300" / "csrc" / "vt_builtins.h"]
OUT = HERE / "_build" / "libvt_oracle.so"


SANITIZED = HERE / "_build" / "libvt_oracle_asan.so"


def build(force: bool = False, sanitize: bool = False) -> Path:
    """The oracle library; with sanitize, a separate build instrumented with
    AddressSanitizer and UndefinedBehaviorSanitizer (errors abort), loaded
    only by the sanitizer test with libasan preloaded."""
    out = SANITIZED if sanitize else OUT
    if not force and out.exists() and all(p.stat().st_mtime <= out.stat().st_mtime for p in [SRC, *HDRS, Path(__file__)]):
        return out
    out.parent.mkdir(parents=True, exist_ok=True)
    tmp = out.with_suffix(".so.tmp")
    flags = ["-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer"] \
        if sanitize else ["-O2"]
    cmd = [os.environ.get("CXX", "g++"), *flags, "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-pthread", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
