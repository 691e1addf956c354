"""Malformed input to the library's host decoders (no GPU): .vox, OBJ, PFM
and Radiance HDR files mutated at random (truncated, bytes flipped, chunk
sizes and dimensions replaced by extreme values) must either decode to
consistent arrays or fail with a status code and a message, never crash or
write past the caller's buffers.  The mutation loop runs in a child process
so that a crash shows up as its exit status; the caller's output buffers
carry guard bytes that are checked after every call."""
import ast
import os
import subprocess
import sys
import textwrap

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = textwrap.dedent(r'''
    import ctypes as C, struct, sys
    import numpy as np
    sys.path.insert(0, ROOT); sys.path.insert(0, HERE)
    from voxeltoy_gb300 import _lib as L
    from test_formats import vox_file, chunk, rgbe, rle_scanline
    lib = L.load()
    GUARD = 64

    def guarded(nbytes):
        buf = np.full(nbytes + 2 * GUARD, 0xA5, np.uint8)
        return buf, buf[GUARD:GUARD + nbytes]

    def intact(buf):
        return (buf[:GUARD] == 0xA5).all() and (buf[-GUARD:] == 0xA5).all()

    def vox(b):
        res = (C.c_int32 * 3)()
        n = C.c_int32()
        if lib.vt_vox_decode(b, len(b), res, None, 0, None, C.byref(n)) != 0:
            return "err"
        nvox = res[0] * res[1] * res[2]
        assert min(res) > 0 and 0 <= n.value <= 255
        if nvox > (1 << 26):
            return "big"
        g, view = guarded(nvox)
        pal, pview = guarded(max(n.value, 1) * C.sizeof(L.Material))
        rc = lib.vt_vox_decode(b, len(b), res, view.ctypes.data_as(C.c_void_p), nvox,
                               pview.ctypes.data_as(C.c_void_p), C.byref(n))
        assert intact(g) and intact(pal)
        if rc == 0:
            assert int(view.max(initial=0)) <= n.value
        return "ok" if rc == 0 else "err"

    def obj(b):
        nv, nt = C.c_int64(), C.c_int64()
        if lib.vt_obj_decode(b, len(b), None, 0, None, 0, C.byref(nv), C.byref(nt)) != 0:
            return "err"
        assert nv.value >= 0 and nt.value >= 0
        if nv.value > (1 << 22) or nt.value > (1 << 22):
            return "big"
        v, vview = guarded(12 * max(nv.value, 1))
        i, iview = guarded(12 * max(nt.value, 1))
        cap_v, cap_t = nv.value, nt.value
        rc = lib.vt_obj_decode(b, len(b), vview.ctypes.data_as(C.c_void_p), cap_v,
                               iview.ctypes.data_as(C.c_void_p), cap_t, C.byref(nv), C.byref(nt))
        assert intact(v) and intact(i)
        if rc == 0 and nt.value:
            idx = iview[:12 * nt.value].view(np.uint32)
            assert int(idx.max()) < nv.value
        return "ok" if rc == 0 else "err"

    def image(b):
        w, h = C.c_int32(), C.c_int32()
        if lib.vt_image_decode(b, len(b), None, 0, C.byref(w), C.byref(h)) != 0:
            return "err"
        assert w.value > 0 and h.value > 0
        n = 12 * w.value * h.value
        if n > (1 << 28):
            return "big"
        g, view = guarded(n)
        rc = lib.vt_image_decode(b, len(b), view.ctypes.data_as(C.c_void_p), n, C.byref(w), C.byref(h))
        assert intact(g)
        return "ok" if rc == 0 else "err"

    rng = np.random.default_rng(int(sys.argv[1]))
    seeds = []
    vx = [(int(x), int(y), int(z), int(c)) for x, y, z, c in rng.integers(0, 6, (40, 4)) if c]
    rgba = rng.integers(0, 256, (256, 4))
    seeds.append((vox, vox_file((6, 6, 6), vx, rgba)))
    seeds.append((vox, vox_file((6, 6, 6), vx, version=200, extra=chunk(b"nTRN", b"\x00" * 12))))
    seeds.append((obj, b"v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nf 1 2 3\nf 1/1 2/2 3/3 4/4\nf -1 -2 -3\n"
                       b"f 2//1 3//1 4//1\no shape\nv 2 2 2\nf 5 1 2\n"))
    img = rng.random((5, 7, 3)).astype(np.float32)
    seeds.append((image, b"PF\n7 5\n-1.0\n" + img.astype("<f4").tobytes()))
    seeds.append((image, b"Pf\n7 5\n1.0\n" + img[..., 0].astype(">f4").tobytes()))
    q = rgbe(np.exp(rng.normal(0, 2, (4, 40, 3))))
    head = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 4 +X 40\n"
    seeds.append((image, head + q.tobytes()))
    seeds.append((image, head + b"".join(rle_scanline(q[y]) for y in range(4))))
    extremes = [0, 1, 0x7fffffff, 0x80000000, 0xffffffff, 0x10000, 255, 256]
    counts = {"ok": 0, "err": 0, "big": 0}
    for fn, data in seeds:
        assert fn(data) == "ok"
        for it in range(int(sys.argv[2])):
            b = bytearray(data)
            kind = it % 4
            if kind == 0:
                b = b[:int(rng.integers(0, len(b)))]
            elif kind == 1:
                for _ in range(int(rng.integers(1, 6))):
                    b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
            elif kind == 2 and len(b) >= 8:
                at = int(rng.integers(0, len(b) - 4))
                b[at:at + 4] = struct.pack("<I", extremes[int(rng.integers(0, len(extremes)))])
            else:
                text = bytes(b).replace(b"5", str(int(rng.choice([0, -1, 99999, 2147483647]))).encode(), 1)
                b = bytearray(text)
            counts[fn(bytes(b))] += 1
    print(counts)
''')


def test_decoders_survive_malformed_input(tmp_path):
    script = tmp_path / "fuzz.py"
    script.write_text(f"ROOT = {ROOT!r}\nHERE = {HERE!r}\n" + CHILD)
    r = subprocess.run([sys.executable, str(script), "7", "3000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    counts = ast.literal_eval(r.stdout.strip().splitlines()[-1])
    assert counts["err"] > 2500 and counts["ok"] > 500
