"""Filtered moment maps (VSM, ESM, EVSM, MSM) on the GPU against the oracle.

Both sides make the same choices where the reference's GL path leaves them
to the driver (moments from the depth map, quad differences for dFdx/dFdy,
box mip levels, the 7-tap blur on texel centres, bilinear level-0 reads).
VSM and MSM use only IEEE-rounded FP32 operations and must match bit for
bit; ESM and EVSM go through exp / log, whose CUDA and libm results may
differ by an ulp, so they are compared within 1e-4 (exp(80 x) turns a
one-ulp difference in x into about 1e-5 relative).
"""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes

pytestmark = pytest.mark.gpu

MOMENT_TECHS = [api.GI_TECH_VSM, api.GI_TECH_ESM, api.GI_TECH_EVSM, api.GI_TECH_MSM]
EXACT = {api.GI_TECH_VSM, api.GI_TECH_MSM}


def _frame(ctx, W, S, tech):
    w = scenes.pcss_1080p(width=W, height=W, map_size=S, spheres=24)
    p = gi.ShadowParams.defaults(tech)
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(ctx)
    bufs = gi.allocate_frame(S, S, W, W)
    gi.render_frame(ctx, w.scene, fr, w.map_params, p, W, W, bufs, store_gbuffer=True)
    return w, p, fr, bufs


def _compare(tech, got, ref):
    # MSM's sqrt of a negative discriminant gives NaN, as the reference's
    # arithmetic does; NaN payloads differ between the GPU and libm, so NaN
    # pixels must coincide and the others match
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    g, r = got[~nan], ref[~nan]
    if tech in EXACT:
        n = int((g.view(np.uint32) != r.view(np.uint32)).sum())
        assert n == 0, f"{n} pixels differ"
    else:
        assert np.allclose(g, r, atol=1e-4, rtol=0), float(np.abs(g - r).max())


@pytest.mark.parametrize("tech", MOMENT_TECHS)
@pytest.mark.parametrize("W,S", [(256, 512), (256, 256), (128, 512)])
def test_moment_frame_matches_oracle(cuda_ctx, tech, W, S):
    import torch

    w, p, fr, bufs = _frame(cuda_ctx, W, S, tech)
    torch.cuda.synchronize()
    depth, pos, nrm = bufs.depth.cpu().numpy(), bufs.pos.cpu().numpy(), bufs.nrm.cpu().numpy()
    ref = oracle.visibility(p.to_c(fr), depth, S, S, pos, nrm, W, W)
    got = bufs.vis.cpu().numpy()
    _compare(tech, got, ref)
    geo = pos.reshape(-1, 4)[:, 0] != 0
    assert (ref[geo] == 1.0).sum() > 100, "lit receivers"
    assert (ref[geo] < 0.9).sum() > 100, "shadowed receivers"
    # the separate visibility pass gives the same image as the fused frame
    vis2 = torch.empty_like(bufs.vis)
    gi.compute_visibility(cuda_ctx, p, fr, bufs.depth, S, S, bufs.pos, bufs.nrm, vis2, W, W)
    torch.cuda.synchronize()
    assert np.array_equal(vis2.cpu().numpy().view(np.uint32), got.view(np.uint32))  # same device, same bits


def test_moment_reference_window_1024_over_2048(cuda_ctx):
    """ShadowMapping's own configuration: 1024^2 window over a 2048^2 map."""
    import torch

    tech = api.GI_TECH_VSM
    w, p, fr, bufs = _frame(cuda_ctx, 1024, 2048, tech)
    torch.cuda.synchronize()
    ref = oracle.visibility(p.to_c(fr), bufs.depth.cpu().numpy(), 2048, 2048, bufs.pos.cpu().numpy(),
                            bufs.nrm.cpu().numpy(), 1024, 1024)
    _compare(tech, bufs.vis.cpu().numpy(), ref)
    soft = ((ref > 0.25) & (ref < 1.0)).sum()
    assert soft > 1000, soft


@pytest.mark.parametrize("W,H,S", [(256, 128, 512), (256, 256, 384), (256, 256, 8192)])
def test_moment_shapes_are_checked(cuda_ctx, W, H, S):
    import torch

    p = gi.ShadowParams.defaults(api.GI_TECH_VSM)
    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=4)
    fr = gi.frame_setup(w.light, w.camera)
    depth = torch.ones(S * S, device="cuda")
    pos = torch.zeros(W * H * 4, device="cuda")
    vis = torch.empty(W * H, device="cuda")
    with pytest.raises(gi.GIError):
        gi.compute_visibility(cuda_ctx, p, fr, depth, S, S, pos, pos, vis, W, H)
