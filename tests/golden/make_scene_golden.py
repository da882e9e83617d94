"""Regenerates tests/golden/scene_pin.npz from the reference's own scene C++.

Builds oracle/_ref/libscene_ref_shadowmapping.so and
libscene_ref_shadowvolumes.so (oracle/ref_scene_pin.cpp linked with the
reference's unmodified SceneLoader.cpp, Mesh.cpp, OBJLoader.cpp and, for
ShadowVolumes, ShadowVolume.cpp) and records:

  * for each loadable Configs file (Dragon, Teapot, Raptor, Door) and each of
    the two apps' loaders: vertex and triangle counts, SHA-256 digests of the
    point, normal and index arrays SceneLoader::load leaves in the Mesh, and
    the camera / light vectors and depth threshold it parsed;
  * Door's whole mesh (points, normals, indices) and the triangles
    ShadowVolume::build makes of it for two lights, one per winding pattern
    in use, resolved through its index buffer (float32 [6T, 3, 3]).

The product's loader (gi_scene_load_config), the oracle's and the product's
volume geometry (or_shadow_volume_geometry, gi_shadow_volume_geometry) must
reproduce these bit for bit (tests/test_scene_pin.py,
tests/test_gpu_volume_geometry.py).  Needs the reference tree; the archive is
committed.

Run:  python tests/golden/make_scene_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle.build_oracle import REFERENCE_ROOT, build_scene_ref  # noqa: E402

OUT = os.path.join(HERE, "scene_pin.npz")
CONFIGS = ("Dragon", "Teapot", "Raptor", "Door")
APPS = ("ShadowMapping", "ShadowVolumes")
VOLUME_LIGHTS = {"le": None, "side": (-30.0, 12.0, 25.0)}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    if len(build_scene_ref()) != len(APPS):
        raise SystemExit("the reference's scene sources are not available here")
    rec = {}
    for name in CONFIGS:
        cfg = os.path.join(REFERENCE_ROOT, "Configs", name + ".txt")
        for app in APPS:
            p, n, ix, views = oracle.ref_load_config(cfg, REFERENCE_ROOT, app)
            key = f"{name}_{app}"
            rec[key + "_counts"] = np.array([p.shape[0], ix.shape[0]], np.int64)
            rec[key + "_sha"] = np.array([digest(p), digest(n), digest(ix)])
            rec[key + "_views"] = views
    p, n, ix, views = oracle.ref_load_config(os.path.join(REFERENCE_ROOT, "Configs", "Door.txt"), REFERENCE_ROOT,
                                             "ShadowVolumes")
    rec["door_points"], rec["door_normals"], rec["door_indices"] = p, n, ix
    for tag, light in VOLUME_LIGHTS.items():
        L = views[6:9].copy() if light is None else np.array(light, np.float32)
        qp, qi = oracle.ref_shadow_volume_build(p, n, ix, L, 100)
        rec[f"door_volume_{tag}_light"] = L
        rec[f"door_volume_{tag}"] = qp[qi.reshape(-1)].reshape(-1, 3, 3)
    np.savez_compressed(OUT, **rec)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
