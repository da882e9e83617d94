"""Regenerates tests/golden/glm_pin.json from the reference's own glm.

Builds oracle/_ref/glm_pin (ref_glm_pin.cpp compiled against the vendored
glm 0.9.3 of the reference, ShadowMapping/include/glm) and records, as IEEE
bit patterns, the matrices the reference builds for a set of frames, the
rotation matrices of Mesh::rotate and computeNormals' face normals.  The
product's host code must reproduce every value bit for bit
(tests/test_matrices.py).  Needs the reference tree; the JSON is committed.

Run:  python tests/golden/make_glm_golden.py
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.build_oracle import build_ref  # noqa: E402

# (light eye, light at, light fov, light w, h, camera eye, camera at, camera fov, camera w, h)
FRAMES = [
    # the reference's Configs views (le/la, ve/va) with its window and map sizes
    ((10, 130, 100), (0, 0, 0), 45, 2048, 2048, (0, 41, -50), (0, 16, -10), 45, 1024, 1024),
    ((10, 140, 100), (0, 0, 0), 45, 1024, 1024, (0, 41, -50), (0, 16, -10), 45, 1280, 720),
    ((10, 130, 100), (0, 0, 0), 45, 2048, 2048, (0, 41, -57), (0, 16, -17), 45, 640, 480),
    ((0, 43, -50), (0, -17, -17), 45, 2048, 2048, (0, 19, -52), (0, -2, -22), 45, 1024, 1024),
    # the synthetic workloads
    ((4, 8, 4), (0, 0, 0), 60, 1024, 1024, (0, 6, -9), (0, 0.6, 0), 45, 1024, 768),
    ((0, 12, 0), (0, 0, 0), 90, 2048, 2048, (0, 14, -20), (0, 0, 0), 45, 1920, 1080),
    ((7, 7, 0), (0, 0, 0), 90, 4096, 4096, (0, 9, -14), (0, 1.5, 0), 45, 3840, 2160),
]
ROTATIONS = [(90, 0, 0), (-90, 0, 270), (0, 90, 0), (12.5, -33.25, 71.0), (0, 0, 0)]
TRIANGLES = [
    (-1, 1, -1, 1, 1, -1, 1, 1, 1),
    (0.1, 0.2, 0.3, 1.7, -0.4, 2.2, -3.1, 0.9, 0.05),
    (33.647778, 59.807484, 4.662212, 33.322739, 59.872997, 4.617175, 34.018166, 59.610893, 4.713532),
]


def main():
    exe = build_ref()
    if exe is None:
        raise SystemExit("the reference's glm is not available here")
    lines = []
    for f in FRAMES:
        le, la, lfov, lw, lh, ce, ca, cfov, cw, ch = f
        lines.append("F " + " ".join(str(v) for v in (*le, *la, lfov, lw, lh, *ce, *ca, cfov, cw, ch)))
    for r in ROTATIONS:
        lines.append("R " + " ".join(str(v) for v in r))
    for t in TRIANGLES:
        lines.append("N " + " ".join(repr(float(v)) for v in t))
    out = subprocess.run([exe], input="\n".join(lines) + "\n", stdout=subprocess.PIPE, text=True,
                         check=True).stdout
    records = [json.loads(l) for l in out.splitlines() if l.strip()]
    doc = {"inputs": {"frames": FRAMES, "rotations": ROTATIONS, "triangles": TRIANGLES},
           "records": records}
    with open(os.path.join(HERE, "glm_pin.json"), "w") as fh:
        json.dump(doc, fh, indent=1)
    print("wrote", len(records), "records")


if __name__ == "__main__":
    main()
