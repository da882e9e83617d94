"""Scene layer: OBJ reader, Mesh operations and the Configs grammar.

Known answers are derived by hand from the reference's rules
(ShadowMapping/src/IO/OBJLoader.cpp glmFirstPass/SecondPass,
ShadowMapping/src/Mesh.cpp, ShadowMapping/src/IO/SceneLoader.cpp).  The
reference's own Configs / OBJ files are read when the reference tree is
present (CPU suite only).
"""
import os

import numpy as np
import pytest

import globalillumination_gb300 as gi
from globalillumination_gb300 import GIError, _capi as api

from conftest import REFERENCE, has_reference


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_obj_formats_and_fans(tmp_path):
    obj = write(tmp_path, "m.obj", """# comment line
mtllib none.mtl
v 0 0 0 0.5 0.5 0.5
v 1 0 0
v 1 1 0
v 0 1 0
vn 0 0 1
vt 0 0
g group one
usemtl x
f 1 2 3 4
f 1//1 2//1 3//1
f 1/1 3/1 4/1
f -4/1/1 -3/1/1 -2/1/1 -1/1/1
""")
    s = gi.Scene().load_obj(obj).commit()
    p, n, i = s.arrays()
    assert p.shape == (4, 3)
    assert np.array_equal(p[2], [1, 1, 0])
    # quad fans (0,1,2),(0,2,3); the relative indices -4..-1 name vertices 1..4
    expect = [[0, 1, 2], [0, 2, 3], [0, 1, 2], [0, 2, 3], [0, 1, 2], [0, 2, 3]]
    assert i.tolist() == expect


def test_obj_unknown_v_token_is_an_error(tmp_path):
    obj = write(tmp_path, "bad.obj", "v 0 0 0\nvp 1 2 3\nf 1 1 1\n")
    with pytest.raises(GIError) as e:
        gi.Scene().load_obj(obj)
    assert e.value.status == api.GI_ERR_PARSE


def test_obj_missing_file():
    with pytest.raises(GIError) as e:
        gi.Scene().load_obj("/nonexistent/x.obj")
    assert e.value.status == api.GI_ERR_IO


def test_compute_normals_running_average():
    # vertex 0 is shared by a +z face and a +x face: the running average is
    # (n1 * (1 - 1/2) + n2 / 2) evaluated in double and stored as float,
    # never re-normalised.
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, -1]], np.float32)
    s = gi.Scene().object_from_arrays(pts, [[0, 1, 2], [0, 2, 3]]).commit()
    _, n, _ = s.arrays()
    assert np.array_equal(n[1], [0, 0, 1])
    assert np.array_equal(n[3], [-1, 0, 0])
    np.testing.assert_array_equal(n[0], np.array([-0.5, 0.0, 0.5], np.float32))
    assert abs(np.linalg.norm(n[0]) - 0.70710677) < 1e-6


def test_scale_translate_do_not_touch_normals_rotate_does():
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    s = gi.Scene().object_from_arrays(pts, [[0, 1, 2]]).scale(2, 3, 4).translate(1, 1, 1).commit()
    p, n, _ = s.arrays()
    assert np.array_equal(p[1], [3, 1, 1]) and np.array_equal(n[0], [0, 0, 1])
    s2 = gi.Scene().object_from_arrays(pts, [[0, 1, 2]]).rotate(90, 0, 0).commit()
    _, n2, _ = s2.arrays()
    assert abs(n2[0][1] + 1.0) < 1e-6 and abs(n2[0][2]) < 1e-6  # +z rotated about x by 90 deg -> -y


def test_commit_offsets_indices():
    s = gi.Scene()
    s.object_from_arrays(np.eye(3, dtype=np.float32), [[0, 1, 2]]).commit()
    s.object_from_arrays(np.eye(3, dtype=np.float32), [[2, 1, 0]]).commit()
    _, _, i = s.arrays()
    assert i.tolist() == [[0, 1, 2], [5, 4, 3]]
    assert s.info().num_objects == 2


def test_config_grammar(tmp_path):
    write(tmp_path, "tri.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    cfg = write(tmp_path, "scene.txt", """o tri.obj
c 1 0 0
cf tri.obj
m white.png
s 2.0 3.0 4.0
t 1 1 1
+
ve 0.0 41.0 -50.0
vx 0.0 16.0 -10.0
le 10.0 130.0 100.0
la 1.0 2.0 3.0
d 0.000025
ha 0
hb 0.001
""")
    s = gi.Scene.from_config(cfg, str(tmp_path))
    inf = s.info()
    assert inf.num_triangles == 1 and inf.num_objects == 1
    assert list(inf.camera_eye) == [0.0, 41.0, -50.0]
    assert list(inf.camera_at) == [0.0, 16.0, -10.0]  # any 2nd char but 'e' means "at"
    assert list(inf.light_eye) == [10.0, 130.0, 100.0]
    assert list(inf.light_at) == [1.0, 2.0, 3.0]
    assert inf.depth_threshold == np.float32(2.5e-5)
    assert inf.hsm_beta == np.float32(0.001)
    p, _, _ = s.arrays()
    assert np.array_equal(p[1], [3, 1, 1])


def test_config_blank_line_repeats_previous_key(tmp_path):
    # SceneLoader keeps `key` and `value` across lines: a blank line repeats
    # the previous key with the previous value ("s 2 3 4" then a blank line
    # scales again by (4, 4, 4)).
    write(tmp_path, "tri.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    cfg = write(tmp_path, "scene.txt", "o tri.obj\ns 2 3 4\n\n+\n")
    s = gi.Scene.from_config(cfg, str(tmp_path))
    p, _, _ = s.arrays()
    assert np.array_equal(p[1], [8, 0, 0]) and np.array_equal(p[2], [0, 12, 0])


def test_config_blank_line_after_commit_is_refused(tmp_path):
    write(tmp_path, "tri.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    cfg = write(tmp_path, "scene.txt", "o tri.obj\n+\n\nve 0 0 0\n")
    # a final "+" followed by end of file is fine
    write(tmp_path, "ok.txt", "o tri.obj\n+\n")
    assert gi.Scene.from_config(str(tmp_path / "ok.txt"), str(tmp_path)).info().num_triangles == 1
    with pytest.raises(GIError) as e:
        gi.Scene.from_config(cfg, str(tmp_path))
    assert e.value.status == api.GI_ERR_PARSE


def test_config_transform_without_object(tmp_path):
    cfg = write(tmp_path, "scene.txt", "s 1 1 1\n")
    with pytest.raises(GIError) as e:
        gi.Scene.from_config(cfg, str(tmp_path))
    assert e.value.status == api.GI_ERR_PARSE


def test_generators():
    s = gi.Scene().ground(10.0, 0.0)
    _, n, i = s.arrays()
    assert i.shape == (2, 3) and np.allclose(n, [0, 1, 0])
    s = gi.Scene().icosphere(3, 1.0, (0, 0, 0))
    p, n, i = s.arrays()
    assert i.shape == (1280, 3) and p.shape == (642, 3)
    assert np.allclose(np.linalg.norm(p, axis=1), 1.0, atol=1e-6)
    # outward normals
    assert (np.sum(p * n, axis=1) > 0).all()
    s = gi.Scene().uv_sphere(64, 32, 1.0, (0, 1.2, 0))
    p, n, i = s.arrays()
    assert i.shape == (64 * 2 + 64 * 30 * 2, 3)
    assert (np.sum((p - [0, 1.2, 0]) * n, axis=1) > 0).all()
    s = gi.Scene().ground(10.0).icosphere_field(64, 3, (-8, 0.2, -8), (8, 3, 8), 0.2, 1.0, 0x5EED0001)
    assert s.info().num_triangles == 81922
    s2 = gi.Scene().ground(10.0).icosphere_field(64, 3, (-8, 0.2, -8), (8, 3, 8), 0.2, 1.0, 0x5EED0001)
    assert np.array_equal(s.arrays()[0], s2.arrays()[0])  # seeded, deterministic
    d = gi.Scene().displaced_sphere(32, 16, 2.0, 0.3, (0, 0, 0), 7)
    p, _, _ = d.arrays()
    r = np.linalg.norm(p, axis=1)
    assert r.min() >= 2.0 - 0.3 - 1e-5 and r.max() <= 2.0 + 0.3 + 1e-5 and r.std() > 0.01


@pytest.mark.skipif(not has_reference(), reason="reference tree not present")
@pytest.mark.parametrize("name,tris", [("Teapot", 15704 + 2), ("Raptor", None), ("Door", None), ("Dragon", None)])
def test_reference_configs_load(name, tris):
    cfg = os.path.join(REFERENCE, "Configs", name + ".txt")
    s = gi.Scene.from_config(cfg, REFERENCE)
    inf = s.info()
    if tris is not None:
        assert inf.num_triangles == tris
    assert list(inf.camera_eye) == [0.0, 41.0, -50.0]
    assert list(inf.camera_at) == [0.0, 16.0, -10.0]
    assert inf.light_eye[1] in (130.0, 140.0)
    p, n, i = s.arrays()
    assert i.min() >= 0 and i.max() < p.shape[0]
    assert np.isfinite(p).all()


@pytest.mark.skipif(not has_reference(), reason="reference tree not present")
def test_reference_plane_obj_normal_points_down():
    # plane.obj's winding gives a -y face normal from computeNormals; the
    # reference relies on the gl_FrontFacing flip to light it.
    s = gi.Scene().load_obj(os.path.join(REFERENCE, "OBJ", "Teapot", "plane.obj")).commit()
    p, n, i = s.arrays()
    assert p.shape == (4, 3) and i.shape == (2, 3)
    assert np.allclose(n, [0, -1, 0])
