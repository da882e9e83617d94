"""Deferred Phong shading (shadeScene / PhongShading.frag) on the GPU
against the CPU oracle, bit for bit, on a rendered frame."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes


@pytest.mark.gpu
@pytest.mark.parametrize("tech", [api.GI_TECH_PCF, api.GI_TECH_PCSS_POISSON])
def test_phong_matches_oracle(cuda_ctx, tech):
    import torch

    w = scenes.pcss_1080p(width=256, height=144, map_size=512, spheres=16)
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    p = gi.ShadowParams.defaults(tech)
    p.light_radius, p.pcss_min_blocker_depth = 0.25, 0.0
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, p, W, H, bufs, store_gbuffer=True)
    g = torch.Generator().manual_seed(3)
    color = torch.rand((H * W * 4,), generator=g).cuda()
    out = torch.empty(H * W * 4, device="cuda")
    gi.phong_shade(cuda_ctx, p, fr, bufs.pos, bufs.nrm, bufs.vis, W, H, out, color=color)
    torch.cuda.synchronize()
    ref = oracle.phong_shade(p.to_c(fr), bufs.pos.cpu().numpy(), bufs.nrm.cpu().numpy(), bufs.vis.cpu().numpy(),
                             W, H, color.cpu().numpy())
    got = out.cpu().numpy()
    assert int((got.view(np.uint32) != ref.view(np.uint32)).sum()) == 0
