"""Host allocation failures through the C ABI: GI_ERR_OOM, never a crash.

The reference exits when a load fails (ShadowMapping/src/Mesh.cpp:336-340,
OBJLoader.cpp:1315-1319) and has no allocation error path at all.  Here a
failed allocation is injected at each allocation point of a scene-building
sequence in turn (gi_debug_fail_allocation); every call must return either
GI_OK or GI_ERR_OOM, a failed call must leave the scene exactly as it was,
and once the injection is off the same sequence builds the same scene."""
import os

import numpy as np
import pytest

import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api

OBJ = """v 0 0 0
v 1 0 0
v 0 1 0
v 1 1 0
f 1 2 3
f 2 4 3
"""


def _steps(obj_path):
    """The scene-building sequence: (name, call(scene))."""
    return [
        ("ground", lambda s: s.ground(10.0)),
        ("icosphere_field", lambda s: s.icosphere_field(6, 2, (-5, 0.2, -5), (5, 2, 5), 0.3, 1.0, 0x5EED00F1)),
        ("load_obj", lambda s: s.load_obj(obj_path)),
        ("scale", lambda s: s.scale(2.0, 1.0, 2.0)),
        ("commit", lambda s: s.commit()),
        ("uv_sphere", lambda s: s.uv_sphere(12, 6, 1.0, (0, 1, 0))),
    ]


def _snapshot(s):
    p, n, i = s.arrays()
    return p.copy(), n.copy(), i.copy(), s.info().num_objects


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a[:3], b[:3])) and a[3] == b[3]


def test_every_injected_host_failure_returns_oom_and_keeps_the_scene(tmp_path):
    obj = os.path.join(str(tmp_path), "quad.obj")
    with open(obj, "w") as f:
        f.write(OBJ)
    ref = gi.Scene()
    for _, step in _steps(obj):
        step(ref)
    want = _snapshot(ref)
    failures = 0
    try:
        for k in range(40):
            s = gi.Scene()
            gi.debug_fail_allocation(k)
            failed_at = None
            for name, step in _steps(obj):
                before = _snapshot(s)
                try:
                    step(s)
                except gi.GIError as e:
                    assert e.status == api.GI_ERR_OOM, (k, name, e)
                    assert _same(_snapshot(s), before), f"{name} changed the scene although it failed"
                    failed_at = name
                    break
            gi.debug_fail_allocation(-1)
            if failed_at is None:
                assert _same(_snapshot(s), want)  # the countdown outlived the sequence
                break
            failures += 1
    finally:
        gi.debug_fail_allocation(-1)
    assert failures >= 6  # every step allocates at least once
    s = gi.Scene()
    for _, step in _steps(obj):
        step(s)
    assert _same(_snapshot(s), want)


def test_injected_failure_in_config_load(tmp_path):
    obj = os.path.join(str(tmp_path), "quad.obj")
    with open(obj, "w") as f:
        f.write(OBJ)
    cfg = os.path.join(str(tmp_path), "scene.txt")
    with open(cfg, "w") as f:
        f.write("o quad.obj\ns 2 2 2\n+\nve 0 1 -5\nva 0 0 0\nle 3 5 3\nla 0 0 0\n")
    try:
        gi.debug_fail_allocation(0)
        with pytest.raises(gi.GIError) as ei:
            gi.Scene.from_config(cfg, str(tmp_path))
        assert ei.value.status == api.GI_ERR_OOM
    finally:
        gi.debug_fail_allocation(-1)
    s = gi.Scene.from_config(cfg, str(tmp_path))
    assert s.info().num_triangles == 2


def test_injection_rejects_bad_countdown():
    with pytest.raises(gi.GIError):
        gi.debug_fail_allocation(-2)
