"""Scene loading and shadow-volume geometry pinned to the reference's own C++.

tests/golden/scene_pin.npz holds what the reference's SceneLoader / Mesh /
glm.c (ShadowMapping/src/IO/SceneLoader.cpp:11-94, src/Mesh.cpp:47-429,
src/IO/OBJLoader.cpp:1309-1387, and ShadowVolumes' copies) and
ShadowVolume::build (ShadowVolumes/src/ShadowVolume.cpp:15-114) produce,
compiled here from the reference's unmodified sources
(oracle/ref_scene_pin.cpp, tests/golden/make_scene_golden.py).  The
product's config loader and the oracle's volume geometry must match it bit
for bit.  Where the reference tree and its compiled pin are present, the
same comparisons also run live.
"""
import hashlib
import os

import numpy as np
import pytest

import globalillumination_gb300 as gi
import oracle
from conftest import REFERENCE, has_reference

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scene_pin.npz")
CONFIGS = ("Dragon", "Teapot", "Raptor", "Door")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.skipif(not has_reference(), reason="reference tree not present")
@pytest.mark.parametrize("name", CONFIGS)
@pytest.mark.parametrize("app", ["ShadowMapping", "ShadowVolumes"])
def test_config_load_equals_reference_fixture(gold, name, app):
    s = gi.Scene.from_config(os.path.join(REFERENCE, "Configs", name + ".txt"), REFERENCE)
    p, n, ix = s.arrays()
    key = f"{name}_{app}"
    assert [p.shape[0], ix.shape[0]] == gold[key + "_counts"].tolist()
    assert [_digest(p), _digest(n), _digest(ix)] == gold[key + "_sha"].tolist()
    inf = s.info()
    views = np.array(list(inf.camera_eye) + list(inf.camera_at) + list(inf.light_eye) + list(inf.light_at) +
                     [inf.depth_threshold if app == "ShadowMapping" else 0.0], np.float32)
    assert np.array_equal(views.view(np.uint32), gold[key + "_views"].view(np.uint32))


@pytest.mark.skipif(oracle.scene_ref("ShadowMapping") is None, reason="reference scene pin not built")
@pytest.mark.parametrize("name", CONFIGS)
def test_config_load_equals_reference_live(name):
    cfg = os.path.join(REFERENCE, "Configs", name + ".txt")
    p, n, ix, _ = oracle.ref_load_config(cfg, REFERENCE, "ShadowMapping")
    P, N, IX = gi.Scene.from_config(cfg, REFERENCE).arrays()
    assert np.array_equal(P.view(np.uint32), p.view(np.uint32))
    assert np.array_equal(N.view(np.uint32), n.view(np.uint32))
    assert np.array_equal(IX, ix)


@pytest.mark.parametrize("tag", ["le", "side"])
def test_oracle_volume_geometry_equals_reference_fixture(gold, tag):
    p, n, ix = gold["door_points"], gold["door_normals"], gold["door_indices"]
    got = oracle.shadow_volume_geometry(p, n, ix, gold[f"door_volume_{tag}_light"], 100.0)
    want = gold[f"door_volume_{tag}"]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.skipif(oracle.scene_ref("ShadowVolumes") is None, reason="reference ShadowVolumes pin not built")
def test_oracle_volume_geometry_equals_reference_live():
    """A synthetic scene (sphere field + ground, both winding patterns under an
    oblique light) through the reference's ShadowVolume::build and the oracle."""
    s = gi.Scene().ground(10.0).icosphere_field(12, 2, (-6, 0.2, -6), (6, 3, 6), 0.3, 1.0, 0x5EED0042)
    p, n, ix = s.arrays()
    for L in ((0.0, 12.0, 0.0), (-7.5, 4.25, 3.0)):
        L = np.array(L, np.float32)
        qp, qi = oracle.ref_shadow_volume_build(p, n, ix, L, 100)
        want = qp[qi.reshape(-1)].reshape(-1, 3, 3)
        got = oracle.shadow_volume_geometry(p, n, ix, L, 100.0)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
