"""Adaptive (quad-tree) area-light sampling in the CPU oracle.

The oracle runs SoftShadowMapping's adaptiveSampling depth first
(evaluateAreaLightSource / renderAreaLightSource, main.cpp:423-690).  These
tests hold it to what the algorithm must produce: samples on the 17 x 17
grid of the area light, each grid position rendered once, no refinement
without partial pixels, the depth limit, the 1 / (2^level + 1)^2 weights
encoded in the translation's w, and an answer close to the uniform 17 x 17
Monte-Carlo estimate of the same light.
"""
import dataclasses

import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import scenes


def view_mvp_for(light):
    def fn(eye, at):
        v = dataclasses.replace(light, eye=tuple(eye), at=tuple(at))
        f = gi.frame_setup(v, v)
        return f.light_mvp, f.light_mvp_biased
    return fn


def run(w, size, max_level, W, H, lower_accuracy=False):
    p, n, i = w.scene.arrays()
    mp = w.map_params
    cam = gi.frame_setup(w.light, w.camera).camera_mvp
    return oracle.area_light_adaptive(p, n, i, w.light.eye, w.light.at, size, max_level, view_mvp_for(w.light),
                                      mp.width, mp.bias_mode, mp.constant_bias, mp.offset_factor, mp.offset_units,
                                      cam, 0.25, W, H, lower_accuracy=lower_accuracy)


def grid_positions(light, size, eyes):
    # sample eye = light eye + (-size / 2 + size * gx / 16, -size / 2 + size * gy / 16, 0)
    d = (eyes[:, :2] - np.asarray(light.eye[:2], np.float32)) / np.float32(size / 16.0) + 8.0
    return np.rint(d).astype(int), d


@pytest.fixture(scope="module")
def small_scene():
    return scenes.pcss_1080p(width=96, height=54, map_size=256, spheres=8)


def test_structure(small_scene):
    # a light of side 4 over the 96 x 54 view: penumbrae wide enough for the
    # evaluation's 3 x 3 test to ask for refinement
    w, size = small_scene, 4.0
    vis, eyes, levels = run(w, size, 4, 96, 54)
    n = len(levels)
    assert 4 <= n <= 289
    g, d = grid_positions(w.light, size, eyes)
    assert np.abs(d - g).max() < 1e-3, "samples on the 17 x 17 grid"
    assert (g >= 0).all() and (g <= 16).all()
    assert len({tuple(x) for x in g}) == n, "a grid position is rendered once"
    assert set(np.unique(levels)) <= {0.0, 1.0, 2.0, 3.0, 4.0}
    # the four root corners come first (the root's evaluation renders them)
    assert {tuple(x) for x in g[:4]} == {(0, 0), (16, 0), (0, 16), (16, 16)}
    # at always moves with eye
    np.testing.assert_allclose(eyes[:, 3:5] - np.asarray(w.light.at[:2]), eyes[:, :2] - np.asarray(w.light.eye[:2]),
                               atol=1e-5)
    assert n > 4, "the shadowed scene needs refinement"
    geo = vis > 0
    assert ((vis[geo] > 0.25) & (vis[geo] < 1.0)).sum() > 20


def test_depth_limit_zero_keeps_the_root(small_scene):
    vis, eyes, levels = run(small_scene, 4.0, 0, 96, 54)
    assert len(levels) == 4 and (levels == 0).all()
    # four maps weighted 1 / (1 + 1)^2 each: every value is a mean of four hard tests
    vals = np.unique(vis[vis > 0])
    allowed = {np.float32((a * 1.0 + (4 - a) * 0.25) * 0.25 / 1.0) for a in range(5)}
    assert all(any(abs(v - a) < 1e-6 for a in allowed) for v in vals)


def test_point_light_needs_no_refinement(small_scene):
    # a zero-size light puts all four corners at the same point: no pixel is
    # partially lit, so the root is not subdivided
    vis, eyes, levels = run(small_scene, 0.0, 4, 96, 54)
    assert len(levels) == 4


def test_close_to_the_uniform_estimate(small_scene):
    w, size = small_scene, 4.0
    vis, _, _ = run(w, size, 4, 96, 54)
    views = gi.area_light_samples(w.light, size, 17)
    frames = [gi.frame_setup(v, w.camera) for v in views]
    p, n, i = w.scene.arrays()
    mp = w.map_params
    mc = oracle.area_light_visibility(p, n, i, np.stack([f.light_mvp for f in frames]),
                                      np.stack([f.light_mvp_biased for f in frames]), mp.width, mp.bias_mode,
                                      mp.constant_bias, mp.offset_factor, mp.offset_units, frames[0].camera_mvp,
                                      0.25, 96, 54)
    geo = mc > 0
    assert np.abs(vis[geo] - mc[geo]).mean() < 0.05


def test_lower_accuracy_mode(small_scene):
    # adaptiveSamplingLowerAccuracy: the evaluation on a quarter-resolution
    # grid needs wider uniform regions, so it refines no more than the full
    # evaluation; the final pass's 4 x 4 taps give intermediate values
    w, size = small_scene, 4.0
    _, _, full = run(w, size, 4, 96, 54)
    vis, eyes, levels = run(w, size, 4, 96, 54, lower_accuracy=True)
    assert 4 <= len(levels) <= len(full)
    fin = vis[vis > 0]
    assert ((fin > 0.25) & (fin < 1.0)).sum() > 20
