"""RBSSM (SoftShadow/RBSSM.frag) on the GPU against the CPU oracle, bit for
bit: random binary maps that reach every reachable smoothing case, and
rendered scenes at several light radii, map sizes and depth thresholds."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes
from rbssm_fuzz import CASES, case


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(len(CASES)))
def test_rbssm_random_maps_bit_exact(cuda_ctx, k):
    import torch

    p, fr, depth, pos, nrm, S, W, H = case(k)
    ref = oracle.visibility(p.to_c(fr), depth, S, S, pos, nrm, W, H)
    d = torch.from_numpy(depth).cuda()
    dp = torch.from_numpy(pos).cuda()
    dn = torch.from_numpy(nrm).cuda()
    out = torch.full((H * W,), -1.0, device="cuda")
    gi.compute_visibility(cuda_ctx, p, fr, d, S, S, dp, dn, out, W, H)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    n_diff = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
    assert n_diff == 0, f"{n_diff} of {W * H} pixels differ"


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [(512, 12, 0.25, 0.0), (256, 24, 2.0, 2.5e-6), (128, 40, 4.0, 0.0),
                                 (1024, 24, 0.5, 1e-5)])
def test_rbssm_scene_bit_exact(cuda_ctx, cfg):
    import torch

    S, spheres, radius, thr = cfg
    W, H = 320, 180
    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=spheres)
    p = gi.ShadowParams.defaults(api.GI_TECH_RBSSM)
    p.light_radius, p.pcss_min_blocker_depth, p.depth_threshold = radius, 0.0, thr
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, p, W, H, bufs, store_gbuffer=True)
    torch.cuda.synchronize()
    pts, nrm, idx = w.scene.arrays()
    d_ref = oracle.shadow_map(pts, idx, fr.light_mvp, S, S, w.map_params.bias_mode, 0.0,
                              w.map_params.offset_factor, w.map_params.offset_units)
    assert np.array_equal(bufs.depth.cpu().numpy().view(np.uint32), d_ref.view(np.uint32))
    pos, nr = oracle.gbuffer(pts, nrm, idx, fr.camera_mvp, W, H)
    ref = oracle.visibility(p.to_c(fr), d_ref, S, S, pos, nr, W, H)
    got = bufs.vis.cpu().numpy()
    n_diff = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
    assert n_diff == 0, f"{n_diff} pixels differ"
    assert ((ref > 0.25) & (ref < 1.0)).sum() > 100  # penumbrae present
