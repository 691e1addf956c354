"""Writes the golden fixtures of tests/golden from their sources.

reference_examples.json
    The worked examples the reference documents in its own comments: the
    environment CDF of src/renderer/image.cpp:107-154 and the binary search
    of src/shaders/envLight/envMapSample.h:10-21, copied as numbers, plus the
    Philox-4x32-10 known-answer vectors published with the algorithm
    (Salmon et al., SC'11).

oracle_frames.npz
    Per-sample radiance and first hits of three small scenes rendered by the
    CPU oracle, together with every input they need (volume, palette,
    emissive list, environment image, raw camera and settings records), so
    that a GPU test can check the CUDA path against them without the oracle
    and without regenerating the seeded scenes:
      config1    48x40 px crop of the config-1 generator (24^3 spheres,
                 Lambert, white sky), samples 0 and 1
      config2    config-2 generator at 24^3 (fBm, 17-entry palette,
                 emissive voxels, 64x32 sky+sun env, thin lens), sample 0
      reference  every reference quirk on, noise-table RNG, sample 0

Run from the repository root:  python tests/golden/make_golden.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

REFERENCE_EXAMPLES = {
    "cdf_rows": {
        "source": "src/renderer/image.cpp:107-154",
        "rows": [[1, 1, 0, 2, 1, 0, 5], [2, 1, 5, 0, 0, 1, 3], [128, 0, 0, 0, 0, 0, 0]],
        "row0_cdf": [0.0, 0.1, 0.2, 0.2, 0.4, 0.5, 0.5, 1.0],
        "marginal": [0.0, "10/150", "22/150", 1.0],
    },
    "binary_search": {
        "source": "src/shaders/envLight/envMapSample.h:10-21",
        "cdf": [0, 0.1, 0.5, 0.6, 0.75, 0.9, 1.0],
        "queries": [[0.7, 3], [0.0, 0], [0.09, 0], [0.1, 1], [0.5999, 2], [0.6, 3], [0.95, 5], [0.99999, 5]],
    },
    "philox4x32_10": {
        "source": "Salmon, Moraes, Dror, Shaw: Parallel random numbers: as easy as 1, 2, 3 (SC'11), "
                  "known-answer vectors of Philox-4x32-10",
        "cases": [
            {"ctr": [0, 0, 0, 0], "key": [0, 0], "out": [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]},
            {"ctr": [0xFFFFFFFF] * 4, "key": [0xFFFFFFFF] * 2,
             "out": [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]},
            {"ctr": [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], "key": [0xA4093822, 0x299F31D0],
             "out": [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]},
        ],
    },
}


def cases():
    from helpers import reference_config, small_config1, small_config2
    return [("config1", small_config1(edge=24, w=48, h=40, seed=1), (0, 1), False),
            ("config2", small_config2(edge=24, w=40, h=32, seed=2), (0,), False),
            ("reference", reference_config(edge=20, w=32, h=24, seed=3), (0,), True)]


def emissive_list(orc, cfg):
    from voxeltoy_gb300 import _lib as L
    if not cfg.scene_flags & L.VT_SCENE_AUTO_EMISSIVE:
        return np.zeros(0, np.int32)
    lit = [i + 1 for i, m in enumerate(cfg.palette) if sum(m[1]) > 0]
    cand = np.flatnonzero(np.isin(cfg.voxels.ravel(), lit)).astype(np.int32)
    return orc.prune_emissive(cfg.voxels, cand) if cfg.scene_flags & L.VT_SCENE_PRUNE_EMISSIVE else cand


def main():
    from oracle import binding as orc
    with open(os.path.join(HERE, "reference_examples.json"), "w") as f:
        json.dump(REFERENCE_EXAMPLES, f, indent=1)
        f.write("\n")
    out = {}
    noise = orc.noise_table()
    for name, cfg, samples, use_noise in cases():
        em = emissive_list(orc, cfg)
        osc = orc.Scene(cfg.voxels, cfg.palette, em if len(em) else None)
        oenv = orc.Env(cfg.env_rgb) if cfg.env_rgb is not None else orc.Env()
        out[f"{name}/voxels"] = cfg.voxels
        out[f"{name}/palette"] = np.array([[t, *e, *a, r] for t, e, a, r in cfg.palette], np.float32)
        out[f"{name}/emissive"] = em
        out[f"{name}/env"] = cfg.env_rgb if cfg.env_rgb is not None else np.zeros((0, 0, 3), np.float32)
        out[f"{name}/camera"] = np.frombuffer(bytes(cfg.camera), np.uint8)
        out[f"{name}/settings"] = np.frombuffer(bytes(cfg.settings), np.uint8)
        out[f"{name}/size"] = np.array([cfg.width, cfg.height], np.int32)
        out[f"{name}/samples"] = np.array(samples, np.int32)
        for smp in samples:
            rgba, hits, _ = orc.render_samples(cfg.camera, cfg.settings, osc, oenv, cfg.width, cfg.height, smp, 32,
                                               noise=noise if use_noise else None)
            out[f"{name}/rgba{smp}"] = rgba.view(np.uint32)
            out[f"{name}/hits{smp}"] = hits
    np.savez_compressed(os.path.join(HERE, "oracle_frames.npz"), **out)


if __name__ == "__main__":
    main()
