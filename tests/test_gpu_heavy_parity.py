"""The heavy scene at its own size against the oracle.

heavy_2160p: a 1024 x 1024 UV-grid sphere displaced by Perlin noise
(2,095,104 triangles) over a ground quad, 4096^2 light maps, a 3840 x 2160
camera.  For one of its eight lights the light map, the G-buffer and the
PCSS (Poisson 16 + 32, with its min-max tap skipping) and non-conservative
SMSR visibility of gi_render_frame must equal the CPU oracle bit for bit
(ShadowMapping/src/main.cpp:221-274,350-372, PlausibleSoftShadow.frag:
166-194,365-398,556-633, RBSM/NonConservativeSMSR.frag:288-304), and the
shadow-volume stencil counts of the same light at 960 x 540 must equal the
oracle's (ShadowVolumes/src/main.cpp:120-206).
"""
import time

import numpy as np
import pytest

import globalillumination_gb300 as gi
import oracle
from globalillumination_gb300 import _capi as api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def heavy():
    w = scenes.heavy_2160p()
    p, n, i = w.scene.arrays()
    return w, (p, n, i)


def test_heavy_frame_full_size_bit_exact(cuda_ctx, heavy):
    import torch

    w, (p, n, i) = heavy
    S, W, H = w.map_params.width, w.camera.width, w.camera.height
    light = gi.ViewSpec(eye=w.lights[0], at=(0.0, 0.0, 0.0), width=S, height=S, fovy_deg=90.0)
    fr = gi.frame_setup(light, w.camera)
    w.scene.upload(cuda_ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    pcss = gi.ShadowParams.defaults(api.GI_TECH_PCSS_POISSON)
    pcss.light_radius = w.params.light_radius
    pcss.pcss_min_blocker_depth = 0.0
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, pcss, W, H, bufs, store_gbuffer=True)
    smsr = gi.ShadowParams.defaults(api.GI_TECH_SMSR_NONCONSERVATIVE)
    vis_smsr = torch.empty_like(bufs.vis)
    gi.compute_visibility(cuda_ctx, smsr, fr, bufs.depth, S, S, bufs.pos, bufs.nrm, vis_smsr, W, H)
    torch.cuda.synchronize()
    mp = w.map_params
    t0 = time.perf_counter()
    d_ref = oracle.shadow_map(p, i, fr.light_mvp, S, S, mp.bias_mode, mp.constant_bias, mp.offset_factor,
                              mp.offset_units)
    d = bufs.depth.cpu().numpy()
    assert np.array_equal(d.view(np.uint32), d_ref.view(np.uint32)), f"{int((d != d_ref).sum())} texels differ"
    pos_ref, nrm_ref = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    pos, nrm = bufs.pos.cpu().numpy().reshape(pos_ref.shape), bufs.nrm.cpu().numpy().reshape(nrm_ref.shape)
    assert np.array_equal(pos.view(np.uint32), pos_ref.view(np.uint32))
    assert np.array_equal(nrm.view(np.uint32), nrm_ref.view(np.uint32))
    tab = np.concatenate([gi.poisson_table(16).reshape(-1), gi.poisson_table(32).reshape(-1)])
    v_ref = oracle.visibility(pcss.to_c(fr), d_ref, S, S, pos_ref, nrm_ref, W, H, tab)
    v = bufs.vis.cpu().numpy()
    assert np.array_equal(v.view(np.uint32), v_ref.view(np.uint32)), f"PCSS: {int((v != v_ref).sum())} pixels differ"
    s_ref = oracle.visibility(smsr.to_c(fr), d_ref, S, S, pos_ref, nrm_ref, W, H)
    s = vis_smsr.cpu().numpy()
    assert np.array_equal(s.view(np.uint32), s_ref.view(np.uint32)), f"SMSR: {int((s != s_ref).sum())} pixels differ"
    soft = float(((v_ref > 0.25) & (v_ref < 1.0)).mean())
    assert soft > 0.001 and (pos_ref.reshape(-1, 4)[:, 3] == 1.0).mean() > 0.5
    print(f"heavy 2160p oracle checks took {time.perf_counter() - t0:.1f} s; soft fraction {soft:.4f}")


def test_heavy_stencil_counts_960x540_bit_exact(cuda_ctx, heavy):
    import torch

    w, (p, n, i) = heavy
    W, H = 960, 540
    cam = gi.ViewSpec(eye=w.camera.eye, at=w.camera.at, width=W, height=H)
    light = gi.ViewSpec(eye=w.lights[0], at=(0.0, 0.0, 0.0), width=64, height=64)
    fr = gi.frame_setup(light, cam)
    w.scene.upload(cuda_ctx)
    st = torch.empty(W * H, dtype=torch.uint8, device="cuda")
    gi.shadow_volume_counts(cuda_ctx, w.scene, light.eye, fr.camera_mvp, W, H, st)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st_ref, _ = oracle.shadow_volume_counts(p, n, i, light.eye, 100.0, fr.camera_mvp, W, H, api.GI_DEPTH_LEQUAL)
    got = st.cpu().numpy()
    assert np.array_equal(got, st_ref), f"{int((got != st_ref).sum())} stencil values differ"
    assert (st_ref != 0).sum() > 10000
    print(f"heavy 960x540 stencil oracle took {time.perf_counter() - t0:.1f} s")
