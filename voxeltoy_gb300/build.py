"""Build recipe of the CUDA library (libvoxeltoy.so) for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into one
shared library next to this file (``voxeltoy_gb300/_lib/libvoxeltoy.so``).
Multiply-add contraction is disabled on the device (``-fmad=false``) and on
the host (``-ffp-contract=off``) because the renderer's arithmetic is
specified operation by operation.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_lib" / "obj"
LIB = OUT_DIR / "libvoxeltoy.so"
CHECKED_LIB = OUT_DIR / "libvoxeltoy_checked.so"   # bounds-checked kernels (VT_CHECKED)
CLI_SRC = PKG / "host" / "vt_cli.cpp"
CLI = OUT_DIR / "vt_cli"

SOURCES = ["vt_api.cu", "vt_render.cu", "vt_scene.cu", "vt_server.cu", "vt_fixed.cu", "vt_io.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-diag-suppress", "128,550",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (cand == "nvcc" or Path(cand).exists()):
            return cand
    return "nvcc"


def _deps() -> list[Path]:
    return [CSRC / s for s in SOURCES] + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def up_to_date(checked: bool = False) -> bool:
    lib = CHECKED_LIB if checked else LIB
    if not lib.exists():
        return False
    t = lib.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps() + [Path(__file__)])


def build_cli(force: bool = False) -> Path:
    """The C++ host program (host/vt_cli.cpp), linked against libvoxeltoy.so
    with an rpath to it, so that it runs from anywhere."""
    if not force and CLI.exists() and CLI.stat().st_mtime >= max(LIB.stat().st_mtime, CLI_SRC.stat().st_mtime):
        return CLI
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-Wall", "-I", str(INCLUDE), str(CLI_SRC),
           "-o", str(CLI), "-L", str(OUT_DIR), "-lvoxeltoy", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("vt_cli build failed:\n" + r.stdout.decode(errors="replace"))
    return CLI


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile every CUDA source and link libvoxeltoy.so (and the C++ host
    program vt_cli next to it); returns the library's path.  checked: the
    bounds-checked variant libvoxeltoy_checked.so (-DVT_CHECKED), for the
    checked test pass."""
    lib = CHECKED_LIB if checked else LIB
    if not force and up_to_date(checked):
        if not checked:
            build_cli()
        return lib
    obj_dir = BUILD_DIR.with_name("obj_checked") if checked else BUILD_DIR
    obj_dir.mkdir(parents=True, exist_ok=True)
    procs = []
    for src in SOURCES:
        obj = obj_dir / (Path(src).stem + ".o")
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *(["-DVT_CHECKED=1"] if checked else []), "-c", str(CSRC / src),
               "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, _obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src}\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *[str(o) for _s, o, _p in procs], "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, lib)
    if not checked:
        build_cli(force=True)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv))
