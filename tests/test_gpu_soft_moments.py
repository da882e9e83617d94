"""Moment soft shadows (SAVSM, VSSM, ESSM, MSSM) on the GPU against the oracle.

The light-side maps (moment map, summed-area table, min-max levels) and the
visibility of rendered frames, with and without the summed-area table.
SAVSM, VSSM and MSSM use only IEEE-rounded FP32 operations and must match
bit for bit; ESSM's exp goes through CUDA's expf on the GPU and glibc's on
the CPU, which may differ by an ulp, so its maps are compared within a
relative 1e-5 and its visibility within 1e-4 on all but a few pixels (a
one-ulp difference can flip the 0.91 and intensity tests of ESSM).
"""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes
from test_soft_moments_oracle import TECHS, blocker_scene, params

pytestmark = pytest.mark.gpu


def _gpu_map(ctx, p, depth, S, T):
    import torch

    d = torch.from_numpy(np.ascontiguousarray(depth, np.float32).reshape(-1)).cuda()
    out = torch.empty(S * T * 4, device="cuda")
    gi.soft_moment_map(ctx, p, d, S, T, out)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(T, S, 4)


def _compare_maps(tech, got, ref):
    if tech == "essm":
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-30)
    else:
        n = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
        assert n == 0, f"{n} map floats differ"


@pytest.mark.parametrize("sat", [False, True])
@pytest.mark.parametrize("tech", list(TECHS))
@pytest.mark.parametrize("S,T", [(64, 64), (100, 37), (300, 200), (40, 2048), (1024, 1024), (2048, 2048),
                                 (4096, 512)])
def test_moment_map_matches_oracle(cuda_ctx, tech, sat, S, T):
    # square, non-square and non-power-of-two maps (a width that is not a
    # power of two leaves the table short of full prefix sums, as the
    # reference's logf-based iteration count does)
    d = blocker_scene(max(S, T), 31)[:T, :S].copy()
    p = params(tech, sat)
    got = _gpu_map(cuda_ctx, p, d, S, T)
    _compare_maps(tech, got, oracle.soft_moment_map(p.to_c(None), d, S, T))


@pytest.mark.parametrize("S,alpha,beta", [(64, 0.0, 0.0), (256, 0.001, -0.002), (2048, 0.0, 0.0005)])
def test_min_max_levels_match_oracle(cuda_ctx, S, alpha, beta):
    import torch

    d = blocker_scene(S, 37)
    d[5, 7] = 0.0
    p = params("vssm", False, hsm_alpha=alpha, hsm_beta=beta)
    td = torch.from_numpy(d.reshape(-1)).cuda()
    for k in range(0, min(5, int(np.log2(S)))):
        out = torch.empty((S >> k) * (S >> k) * 2, device="cuda")
        gi.hierarchical_shadow_map(cuda_ctx, p, td, S, S, k, out)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(S >> k, S >> k, 2)
        ref = oracle.hierarchical_shadow_map(p.to_c(None), d, S, S, k)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), f"level {k}"


def _frame(ctx, W, H, S, tech, sat, radius):
    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=24)
    p = gi.ShadowParams.defaults(TECHS[tech])
    p.summed_area_table = sat
    p.light_radius = radius
    p.pcss_min_blocker_depth = 0.0
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_frame(ctx, w.scene, fr, w.map_params, p, W, H, bufs, store_gbuffer=True)
    return p, fr, bufs


@pytest.mark.parametrize("sat", [False, True])
@pytest.mark.parametrize("tech", list(TECHS))
@pytest.mark.parametrize("W,H,S", [(256, 144, 512), (320, 180, 1024), (192, 108, 2048)])
def test_frame_matches_oracle(cuda_ctx, tech, sat, W, H, S):
    import torch

    p, fr, bufs = _frame(cuda_ctx, W, H, S, tech, sat, 0.25 if not sat else 0.05)
    torch.cuda.synchronize()
    depth, pos, nrm = bufs.depth.cpu().numpy(), bufs.pos.cpu().numpy(), bufs.nrm.cpu().numpy()
    ref = oracle.visibility(p.to_c(fr), depth, S, S, pos, nrm, W, H)
    got = bufs.vis.cpu().numpy()
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    g, r = got[~nan], ref[~nan]
    if tech == "essm":
        bad = ~np.isclose(g, r, rtol=0, atol=1e-4)
        assert bad.sum() <= max(3, g.size // 2000), f"{int(bad.sum())} pixels differ"
    else:
        n = int((g.view(np.uint32) != r.view(np.uint32)).sum())
        assert n == 0, f"{n} pixels differ"
    geo = pos.reshape(-1, 4)[:, 0] != 0
    assert (ref[geo] == 1.0).sum() > 100, "lit receivers"
    assert (ref[geo] < 1.0).sum() > 20, "shadowed receivers"
    # the separate visibility pass gives the same image as the fused frame
    vis2 = torch.empty_like(bufs.vis)
    gi.compute_visibility(cuda_ctx, p, fr, bufs.depth, S, S, bufs.pos, bufs.nrm, vis2, W, H)
    torch.cuda.synchronize()
    assert np.array_equal(vis2.cpu().numpy().view(np.uint32), got.view(np.uint32))


def test_vssm_shape_is_checked(cuda_ctx):
    import torch

    p = gi.ShadowParams.defaults(api.GI_TECH_VSSM)
    fr = gi.frame_setup(scenes.pcss_1080p(width=64, height=64, map_size=64, spheres=1).light,
                        scenes.pcss_1080p(width=64, height=64, map_size=64, spheres=1).camera)
    pos = torch.zeros(64 * 64 * 4, device="cuda")
    vis = torch.empty(64 * 64, device="cuda")
    for S, T in ((96, 96), (64, 32), (4, 4)):
        depth = torch.ones(S * T, device="cuda")
        with pytest.raises(gi.GIError):
            gi.compute_visibility(cuda_ctx, p, fr, depth, S, T, pos, pos, vis, 64, 64)
    # the other moment soft shadows take any map shape
    p = gi.ShadowParams.defaults(api.GI_TECH_SAVSM)
    depth = torch.ones(96 * 80, device="cuda")
    gi.compute_visibility(cuda_ctx, p, fr, depth, 96, 80, pos, pos, vis, 64, 64)
    torch.cuda.synchronize()
    with pytest.raises(gi.GIError):
        gi.hierarchical_shadow_map(cuda_ctx, p, depth, 96, 80, 1, torch.empty(48 * 40 * 2, device="cuda"))
