"""Matrix code pinned bit for bit against the reference's vendored glm 0.9.3.

tests/golden/glm_pin.json was produced by tests/golden/make_glm_golden.py,
which compiles oracle/ref_glm_pin.cpp against the reference's own glm
headers.  The values depend on the host libm's tanf / sinf / cosf, which is
why these tests run on the host that made the fixture (x86_64 glibc) and are
skipped elsewhere.
"""
import json
import os
import platform
import struct

import numpy as np
import pytest

import globalillumination_gb300 as gi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "glm_pin.json")

pytestmark = pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"),
                                reason="fixture made with x86_64 glibc libm")


def _bits(arr):
    return ["%08x" % struct.unpack("<I", struct.pack("<f", float(v)))[0] for v in np.asarray(arr).reshape(-1)]


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def _frames(golden):
    recs = [r for r in golden["records"] if r["kind"] == "F"]
    return list(zip(golden["inputs"]["frames"], recs))


def test_frame_matrices_bit_exact(golden):
    for inp, rec in _frames(golden):
        le, la, lfov, lw, lh, ce, ca, cfov, cw, ch = inp
        light = gi.ViewSpec(eye=le, at=la, width=lw, height=lh, fovy_deg=lfov)
        cam = gi.ViewSpec(eye=ce, at=ca, width=cw, height=ch, fovy_deg=cfov)
        fr = gi.frame_setup(light, cam)
        assert _bits(fr.light_mvp) == rec["light_mvp"], inp
        assert _bits(fr.light_mvp_biased) == rec["light_mvp_biased"], inp
        assert _bits(fr.camera_mvp) == rec["camera_mvp"], inp
        assert _bits(fr.camera_mv) == rec["camera_mv"], inp
        assert _bits(fr.normal_matrix) == rec["normal_matrix"], inp
        assert _bits(fr.light_position) == rec["light_position"], inp


def test_view_matrices_bit_exact(golden):
    import ctypes as C

    from globalillumination_gb300 import _capi as api

    for inp, rec in _frames(golden):
        le, la, lfov, lw, lh = inp[:5]
        v = gi.ViewSpec(eye=le, at=la, width=lw, height=lh, fovy_deg=lfov).to_c()
        P, V = api.F16(), api.F16()
        api.check(api.load().gi_view_matrices(C.byref(v), P, V), "gi_view_matrices")
        assert _bits(list(P)) == rec["light_proj"]
        assert _bits(list(V)) == rec["light_view"]


def test_mesh_rotate_matrix_bit_exact(golden):
    recs = [r for r in golden["records"] if r["kind"] == "R"]
    for ang, rec in zip(golden["inputs"]["rotations"], recs):
        s = gi.Scene()
        pts = np.eye(3, dtype=np.float32)
        s.object_from_arrays(pts, [[0, 1, 2]]).rotate(*ang).commit()
        p, _, _ = s.arrays()
        t = rec["rotation_t"]  # transpose(Rx Ry Rz), column-major
        # rotating e_k yields column k of Rx Ry Rz = row k of its transpose
        for k in range(3):
            assert _bits(p[k]) == [t[0 * 4 + k], t[1 * 4 + k], t[2 * 4 + k]], (ang, k)


def test_face_normals_bit_exact(golden):
    recs = [r for r in golden["records"] if r["kind"] == "N"]
    for tri, rec in zip(golden["inputs"]["triangles"], recs):
        s = gi.Scene()
        s.object_from_arrays(np.array(tri, np.float32).reshape(3, 3), [[0, 1, 2]]).commit()
        _, n, _ = s.arrays()
        for k in range(3):
            assert _bits(n[k]) == rec["normal"]
