"""Adaptive (quad-tree) area-light ground truth on the GPU against the CPU
oracle: the same samples (eye and at bit for bit, in the same order), the
same levels, and the visibility bit for bit."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import scenes
from test_area_adaptive_oracle import run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,S,size,max_level,spheres,lower",
                         [(96, 54, 256, 4.0, 4, 8, False), (160, 96, 512, 8.0, 4, 16, False),
                          (192, 108, 256, 2.0, 4, 8, False), (128, 72, 512, 6.0, 2, 16, False),
                          (96, 54, 256, 4.0, 0, 8, False), (192, 108, 256, 4.0, 4, 8, True),
                          (150, 90, 512, 8.0, 4, 16, True)])
def test_adaptive_matches_oracle(cuda_ctx, W, H, S, size, max_level, spheres, lower):
    import torch

    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=spheres)
    w.scene.upload(cuda_ctx)
    cam = gi.frame_setup(w.light, w.camera).camera_mvp
    vis = torch.full((W * H,), -1.0, device="cuda")
    _, views, levels = gi.area_light_adaptive(cuda_ctx, w.scene, w.light, size, w.map_params, cam, 0.25, W, H, vis,
                                              max_level=max_level, lower_accuracy=lower)
    torch.cuda.synchronize()
    ref, eyes, ref_levels = run(w, size, max_level, W, H, lower_accuracy=lower)
    got_eyes = np.array([list(v.eye) + list(v.at) for v in views], np.float32)
    assert got_eyes.shape == eyes.shape
    np.testing.assert_array_equal(got_eyes.view(np.uint32), eyes.view(np.uint32))
    np.testing.assert_array_equal(levels, ref_levels)
    got = vis.cpu().numpy()
    n = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
    assert n == 0, f"{n} pixels differ"


def test_adaptive_rejects_bad_input(cuda_ctx):
    import torch

    w = scenes.pcss_1080p(width=64, height=64, map_size=128, spheres=2)
    w.scene.upload(cuda_ctx)
    cam = gi.frame_setup(w.light, w.camera).camera_mvp
    vis = torch.empty(64 * 64, device="cuda")
    for kw in (dict(max_level=5), dict(max_level=-1)):
        with pytest.raises(gi.GIError):
            gi.area_light_adaptive(cuda_ctx, w.scene, w.light, 4.0, w.map_params, cam, 0.25, 64, 64, vis, **kw)
    with pytest.raises(gi.GIError):
        gi.area_light_adaptive(cuda_ctx, w.scene, w.light, -1.0, w.map_params, cam, 0.25, 64, 64, vis)
    mp = gi.MapParams(128, 64)
    with pytest.raises(gi.GIError):
        gi.area_light_adaptive(cuda_ctx, w.scene, w.light, 4.0, mp, cam, 0.25, 64, 64, vis)
