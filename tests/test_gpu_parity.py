"""CUDA path vs CPU oracle, through the C ABI, on seeded synthetic scenes.

Depth maps, G-buffers and stencil counts must be bit-identical.  Visibility
must match within 1e-3 absolute (the bar the reference's float passes are
held to); the kernels perform the oracle's FP32 operations in the same order,
so the tests also report how many pixels differ at all and expect none.
"""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes

pytestmark = pytest.mark.gpu

VIS_TOL = 1e-3


def _torch():
    import torch

    return torch


def _run_frame(ctx, w, W, H, S, params=None):
    torch = _torch()
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_shadow_map(ctx, w.scene, w.map_params, fr.light_mvp, bufs.depth)
    gi.render_gbuffer(ctx, w.scene, fr.camera_mvp, W, H, bufs.pos, bufs.nrm)
    gi.compute_visibility(ctx, params or w.params, fr, bufs.depth, S, S, bufs.pos, bufs.nrm, bufs.vis, W, H)
    torch.cuda.synchronize()
    return fr, bufs


def _small_c1(W=256, H=192, S=256):
    w = scenes.hard_pcf_1024(width=W, height=H, map_size=S)
    return w


def _small_c2(W=320, H=180, S=512, spheres=12):
    return scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=spheres)


@pytest.mark.parametrize("bias_mode", [api.GI_BIAS_NONE, api.GI_BIAS_CONSTANT, api.GI_BIAS_POLYGON_OFFSET])
@pytest.mark.parametrize("size", [(256, 256), (250, 170), (1, 1), (17, 33)])
def test_depth_map_bit_exact(cuda_ctx, bias_mode, size):
    torch = _torch()
    w = _small_c1()
    mw, mh = size
    w.map_params.width, w.map_params.height = mw, mh
    w.map_params.bias_mode = bias_mode
    w.light.width, w.light.height = mw, mh
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    depth = torch.empty(mw * mh, dtype=torch.float32, device="cuda")
    gi.render_shadow_map(cuda_ctx, w.scene, w.map_params, fr.light_mvp, depth)
    torch.cuda.synchronize()
    p, n, i = w.scene.arrays()
    ref = oracle.shadow_map(p, i, fr.light_mvp, mw, mh, bias_mode, w.map_params.constant_bias,
                            w.map_params.offset_factor, w.map_params.offset_units)
    got = depth.cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), \
        f"{int((got != ref).sum())} texels differ"


@pytest.mark.parametrize("dims", [(256, 192), (250, 170), (1920 // 4, 1080 // 4)])
def test_gbuffer_bit_exact(cuda_ctx, dims):
    W, H = dims
    w = _small_c2(W, H)
    fr, bufs = _run_frame(cuda_ctx, w, W, H, w.map_params.width)
    p, n, i = w.scene.arrays()
    pos_ref, nrm_ref = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    pos, nrm = bufs.pos.cpu().numpy(), bufs.nrm.cpu().numpy()
    assert np.array_equal(pos.view(np.uint32), pos_ref.view(np.uint32)), \
        f"{int((pos != pos_ref).sum())} position floats differ"
    assert np.array_equal(nrm.view(np.uint32), nrm_ref.view(np.uint32)), \
        f"{int((nrm != nrm_ref).sum())} normal floats differ"


TECHS = [api.GI_TECH_HARD, api.GI_TECH_PCF, api.GI_TECH_PCF_TRICUBIC, api.GI_TECH_PCSS_GRID,
         api.GI_TECH_PCSS_POISSON, api.GI_TECH_SMSR_CONSERVATIVE, api.GI_TECH_SMSR_NONCONSERVATIVE,
         api.GI_TECH_RPCF_CONSERVATIVE, api.GI_TECH_RPCF_SMSR, api.GI_TECH_RSMSS, api.GI_TECH_HARD_SOFTAPP,
         api.GI_TECH_RBSSM]


def _vis_params(w, tech):
    p = gi.ShadowParams.defaults(tech)
    p.kernel_order = 3
    p.light_radius = w.params.light_radius
    p.pcss_min_blocker_depth = w.params.pcss_min_blocker_depth
    p.depth_threshold = 2.5e-6
    return p


@pytest.mark.parametrize("tech", TECHS)
@pytest.mark.parametrize("scene", ["c1", "c2"])
def test_visibility_matches_oracle(cuda_ctx, tech, scene):
    w = _small_c1() if scene == "c1" else _small_c2()
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    params = _vis_params(w, tech)
    fr, bufs = _run_frame(cuda_ctx, w, W, H, S, params)
    # Check the visibility pass on the GPU's own inputs, then the whole chain.
    depth = bufs.depth.cpu().numpy()
    pos, nrm = bufs.pos.cpu().numpy(), bufs.nrm.cpu().numpy()
    tab = np.concatenate([gi.poisson_table(params.poisson_blocker_taps).reshape(-1),
                          gi.poisson_table(params.poisson_filter_taps).reshape(-1)])
    ref = oracle.visibility(params.to_c(fr), depth, S, S, pos, nrm, W, H, tab)
    got = bufs.vis.cpu().numpy()
    assert np.allclose(got, ref, atol=VIS_TOL, rtol=0, equal_nan=True)
    n_diff = int((got.view(np.uint32) != ref.view(np.uint32)).sum())
    assert n_diff == 0, f"{n_diff} pixels differ in their last bits"


def test_full_chain_c1_1024(cuda_ctx):
    """hard_pcf_1024 at its full size: 1024^2 map, 1024 x 768, 3x3 PCF."""
    w = scenes.hard_pcf_1024()
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    fr, bufs = _run_frame(cuda_ctx, w, W, H, S)
    p, n, i = w.scene.arrays()
    d_ref = oracle.shadow_map(p, i, fr.light_mvp, S, S, w.map_params.bias_mode, w.map_params.constant_bias)
    pos_ref, nrm_ref = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    vis_ref = oracle.visibility(w.params.to_c(fr), d_ref, S, S, pos_ref, nrm_ref, W, H)
    assert np.array_equal(bufs.depth.cpu().numpy().view(np.uint32), d_ref.view(np.uint32))
    assert np.array_equal(bufs.pos.cpu().numpy().view(np.uint32), pos_ref.view(np.uint32))
    got = bufs.vis.cpu().numpy()
    assert np.allclose(got, vis_ref, atol=VIS_TOL, rtol=0)
    assert int((got != vis_ref).sum()) == 0
    # the scene has both lit and shadowed receivers
    assert (vis_ref == 1.0).sum() > 1000 and (vis_ref == 0.25).sum() > 1000


def test_full_chain_pcss_1080p(cuda_ctx):
    """pcss_1080p at its full size: 81,922 triangles, 2048^2 map, 1920 x 1080, PCSS 16/32."""
    w = scenes.pcss_1080p()
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    fr, bufs = _run_frame(cuda_ctx, w, W, H, S)
    p, n, i = w.scene.arrays()
    assert i.shape[0] == 81922
    mp = w.map_params
    d_ref = oracle.shadow_map(p, i, fr.light_mvp, S, S, mp.bias_mode, mp.constant_bias, mp.offset_factor,
                              mp.offset_units)
    assert np.array_equal(bufs.depth.cpu().numpy().view(np.uint32), d_ref.view(np.uint32))
    pos_ref, nrm_ref = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    assert np.array_equal(bufs.pos.cpu().numpy().view(np.uint32), pos_ref.view(np.uint32))
    assert np.array_equal(bufs.nrm.cpu().numpy().view(np.uint32), nrm_ref.view(np.uint32))
    tab = np.concatenate([gi.poisson_table(16).reshape(-1), gi.poisson_table(32).reshape(-1)])
    vis_ref = oracle.visibility(w.params.to_c(fr), d_ref, S, S, pos_ref, nrm_ref, W, H, tab)
    got = bufs.vis.cpu().numpy()
    assert np.allclose(got, vis_ref, atol=VIS_TOL, rtol=0)
    assert int((got != vis_ref).sum()) == 0
    # soft shadows exist: fractional visibility values
    frac = ((vis_ref > 0.25) & (vis_ref < 1.0)).sum()
    assert frac > 1000, frac


@pytest.mark.parametrize("depth_func", [api.GI_DEPTH_LESS, api.GI_DEPTH_LEQUAL])
@pytest.mark.parametrize("dims", [(160, 120), (203, 97)])
def test_shadow_volume_counts_bit_exact(cuda_ctx, depth_func, dims):
    torch = _torch()
    W, H = dims
    s = gi.Scene()
    s.ground(10.0, 0.0)
    s.uv_sphere(24, 12, 1.0, (0.0, 1.5, 0.0))
    s.icosphere(1, 0.6, (2.0, 1.0, 1.0))
    cam = gi.ViewSpec(eye=(0.0, 7.0, -10.0), at=(0.0, 0.5, 0.0), width=W, height=H)
    light = gi.ViewSpec(eye=(3.0, 9.0, 2.0), at=(0.0, 0.0, 0.0), width=64, height=64)
    fr = gi.frame_setup(light, cam)
    s.upload(cuda_ctx)
    st = torch.empty(W * H, dtype=torch.uint8, device="cuda")
    dp = torch.empty(W * H, dtype=torch.float32, device="cuda")
    gi.shadow_volume_counts(cuda_ctx, s, light.eye, fr.camera_mvp, W, H, st, dp, depth_func=depth_func)
    torch.cuda.synchronize()
    p, n, i = s.arrays()
    st_ref, dp_ref = oracle.shadow_volume_counts(p, n, i, light.eye, 100.0, fr.camera_mvp, W, H, depth_func)
    assert np.array_equal(dp.cpu().numpy().view(np.uint32), dp_ref.view(np.uint32))
    got = st.cpu().numpy()
    assert np.array_equal(got, st_ref), f"{int((got != st_ref).sum())} stencil values differ"
    assert (st_ref != 0).sum() > 0 and (st_ref == 0).sum() > 0


@pytest.mark.parametrize("light_eye", [(4.9, 7.0, 0.0), (-2.0, 6.0, -5.0)])
def test_shadow_volume_slivers_bit_exact(cuda_ctx, light_eye):
    """A displaced sphere (the heavy scene's shape at a small size): its
    extruded sides are long slivers, drawn by the row-span path."""
    torch = _torch()
    W, H = 320, 240
    s = gi.Scene()
    s.ground(10.0, 0.0)
    s.displaced_sphere(40, 20, 2.0, 0.3, (0.0, 2.6, 0.0), 0x5EED0004)
    cam = gi.ViewSpec(eye=(0.0, 9.0, -14.0), at=(0.0, 1.5, 0.0), width=W, height=H)
    light = gi.ViewSpec(eye=light_eye, at=(0.0, 0.0, 0.0), width=64, height=64)
    fr = gi.frame_setup(light, cam)
    s.upload(cuda_ctx)
    st = torch.empty(W * H, dtype=torch.uint8, device="cuda")
    gi.shadow_volume_counts(cuda_ctx, s, light.eye, fr.camera_mvp, W, H, st)
    torch.cuda.synchronize()
    p, n, i = s.arrays()
    st_ref, _ = oracle.shadow_volume_counts(p, n, i, light.eye, 100.0, fr.camera_mvp, W, H, api.GI_DEPTH_LEQUAL)
    got = st.cpu().numpy()
    assert np.array_equal(got, st_ref), f"{int((got != st_ref).sum())} stencil values differ"
    assert (st_ref != 0).sum() > 1000


@pytest.mark.parametrize("tech", [api.GI_TECH_PCF, api.GI_TECH_PCSS_POISSON, api.GI_TECH_SMSR_NONCONSERVATIVE,
                                  api.GI_TECH_RSMSS])
@pytest.mark.parametrize("store", [False, True])
def test_fused_frame_equals_passes(cuda_ctx, tech, store):
    """gi_render_frame (resolve + visibility in one kernel) == the three passes."""
    torch = _torch()
    w = _small_c2(W=333, H=190, S=512)
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    params = _vis_params(w, tech)
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    a = gi.allocate_frame(S, S, W, H)
    b = gi.allocate_frame(S, S, W, H)
    gi.render_frame_passes(cuda_ctx, w.scene, fr, w.map_params, params, W, H, a)
    b.pos.fill_(-3.0)
    b.nrm.fill_(-3.0)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, params, W, H, b, store_gbuffer=store)
    torch.cuda.synchronize()
    assert torch.equal(a.depth.view(torch.int32), b.depth.view(torch.int32))
    assert torch.equal(a.vis.view(torch.int32), b.vis.view(torch.int32))
    if store:
        assert torch.equal(a.pos.view(torch.int32), b.pos.view(torch.int32))
        assert torch.equal(a.nrm.view(torch.int32), b.nrm.view(torch.int32))
    else:
        assert bool((b.pos == -3.0).all())


def test_empty_scene(cuda_ctx):
    torch = _torch()
    s = gi.Scene()
    s.upload(cuda_ctx)
    light = gi.ViewSpec(eye=(0, 10, 0), at=(0, 0, 0), width=64, height=64)
    cam = gi.ViewSpec(eye=(0, 5, -5), at=(0, 0, 0), width=48, height=32)
    fr = gi.frame_setup(light, cam)
    bufs = gi.allocate_frame(64, 64, 48, 32)
    gi.render_frame(cuda_ctx, s, fr, gi.MapParams(64, 64), gi.ShadowParams.defaults(api.GI_TECH_PCF), 48, 32, bufs,
                    store_gbuffer=True)
    torch.cuda.synchronize()
    assert (bufs.depth.cpu().numpy() == 1.0).all()
    assert (bufs.vis.cpu().numpy() == 0.0).all()
    assert (bufs.pos.cpu().numpy().reshape(-1, 4) == np.array([0, 0, 0, 1], np.float32)).all()
