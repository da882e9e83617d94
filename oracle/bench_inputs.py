"""Inputs of the CPU baseline (test infrastructure only).

The timed CPU restatement in bench.py's reference arm must load no product
code, so the pcss_1080p workload it renders is read from a committed archive
(oracle/pcss_1080p_inputs.npz): the scene arrays (ground + 64 seeded
icospheres, 81,922 triangles), the light and camera matrices, the map
parameters, the visibility parameter block as the C ABI lays it out
(gi_vis_params) and the Poisson-disk table.  `make()` writes the archive from
the product's own generators; tests/test_bench_inputs.py checks that the
archive still equals what the product generates, so both arms of the
benchmark render the same frame.

Regenerate:  python -m oracle.bench_inputs
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "pcss_1080p_inputs.npz")


def make(path: str = PATH) -> dict:
    """Builds the archive from the product's generators (needs libgishadow.so)."""
    import globalillumination_gb300 as gi
    from globalillumination_gb300 import scenes

    w = scenes.pcss_1080p()
    fr = gi.frame_setup(w.light, w.camera)
    p, n, i = w.scene.arrays()
    mp = w.map_params
    vis = w.params.to_c(fr)
    tab = np.concatenate([gi.poisson_table(w.params.poisson_blocker_taps).reshape(-1),
                          gi.poisson_table(w.params.poisson_filter_taps).reshape(-1)])
    rec = {
        "points": p, "normals": n, "indices": i,
        "light_mvp": np.asarray(fr.light_mvp, np.float32), "camera_mvp": np.asarray(fr.camera_mvp, np.float32),
        "map": np.array([mp.width, mp.bias_mode], np.int32),
        "map_bias": np.array([mp.constant_bias, mp.offset_factor, mp.offset_units], np.float32),
        "camera": np.array([w.camera.width, w.camera.height], np.int32),
        "vis_params": np.frombuffer(bytes(vis), np.uint8).copy(),
        "poisson": tab.astype(np.float32),
    }
    if path:
        np.savez_compressed(path, **rec)
    return rec


class Inputs:
    """The archive's contents, with the visibility block as a C buffer for the oracle."""

    def __init__(self, path: str = PATH):
        z = np.load(path)
        self.points, self.normals, self.indices = z["points"], z["normals"], z["indices"]
        self.light_mvp, self.camera_mvp = z["light_mvp"], z["camera_mvp"]
        self.S, self.bias_mode = (int(v) for v in z["map"])
        self.constant_bias, self.offset_factor, self.offset_units = (float(v) for v in z["map_bias"])
        self.W, self.H = (int(v) for v in z["camera"])
        self.vis_params = C.create_string_buffer(z["vis_params"].tobytes(), len(z["vis_params"]))
        self.poisson = z["poisson"]


if __name__ == "__main__":
    make()
    print("wrote", PATH, os.path.getsize(PATH), "bytes")
