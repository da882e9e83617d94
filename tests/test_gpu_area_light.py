"""Area-light ground truth (renderMonteCarlo + AccurateSoftShadow.frag) on
the GPU against the CPU oracle, bit for bit, for several sample grids and
map sizes (waves of up to 16 maps, so 25 samples exercise two waves)."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes


@pytest.mark.gpu
@pytest.mark.parametrize("n_side,S,size", [(3, 256, 0.5), (5, 128, 1.0), (5, 512, 0.25)])
def test_area_light_matches_oracle(cuda_ctx, n_side, S, size):
    import torch

    W, H = 160, 96
    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=16)
    views = gi.area_light_samples(w.light, size, n_side)
    frames = [gi.frame_setup(v, w.camera) for v in views]
    w.scene.upload(cuda_ctx)
    vis = torch.full((W * H,), -1.0, device="cuda")
    gi.area_light_visibility(cuda_ctx, w.scene, views, w.map_params, frames[0].camera_mvp, 0.25, W, H, vis)
    torch.cuda.synchronize()
    p, n, i = w.scene.arrays()
    mp = w.map_params
    ref = oracle.area_light_visibility(p, n, i, np.stack([f.light_mvp for f in frames]),
                                       np.stack([f.light_mvp_biased for f in frames]), S, mp.bias_mode,
                                       mp.constant_bias, mp.offset_factor, mp.offset_units, frames[0].camera_mvp,
                                       0.25, W, H)
    got = vis.cpu().numpy()
    n_diff = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
    assert n_diff == 0, f"{n_diff} pixels differ"
    assert ((ref > 0.25) & (ref < 1.0)).sum() > 20  # penumbrae present


@pytest.mark.gpu
def test_area_light_rejects_bad_input(cuda_ctx):
    import torch

    w = scenes.pcss_1080p(width=64, height=32, map_size=64, spheres=2)
    w.scene.upload(cuda_ctx)
    vis = torch.empty(64 * 32, device="cuda")
    views = gi.area_light_samples(w.light, 0.5, 3)
    fr = gi.frame_setup(views[0], w.camera)
    with pytest.raises(gi.GIError):
        gi.area_light_visibility(cuda_ctx, w.scene, [], w.map_params, fr.camera_mvp, 0.25, 64, 32, vis)
    with pytest.raises(gi.GIError):
        gi.area_light_visibility(cuda_ctx, w.scene, views, gi.MapParams(64, 32), fr.camera_mvp, 0.25, 64, 32, vis)
