"""Batched frames (gi_batch_*): every light's visibility image equals the
single-frame path (gi_render_frame) bit for bit, for every stream count and
tier threshold, and one light per batch is checked against the CPU oracle."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes


def _small_batch(n=6, W=192, H=108):
    return scenes.batched_720p(scenes=n, width=W, height=H, tri_min=200, tri_max=20_000,
                               map_sides=(128, 256, 512), max_lights=3, seed=scenes.SEED_BASE + 92)


def _upload(ctx, frames):
    for f in frames:
        f.scene.upload(ctx)


def _outputs(frames):
    import torch

    return [torch.full((len(f.lights), f.camera.height, f.camera.width), -7.0, device="cuda") for f in frames]


def _single(ctx, f, l):
    import torch

    fr = gi.frame_setup(f.lights[l], f.camera)
    mp = f.maps[l]
    bufs = gi.allocate_frame(mp.width, mp.height, f.camera.width, f.camera.height)
    gi.render_frame(ctx, f.scene, fr, mp, f.params, f.camera.width, f.camera.height, bufs)
    torch.cuda.synchronize()
    return bufs.vis.cpu().numpy().reshape(f.camera.height, f.camera.width), bufs.depth.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("streams", [1, 3, 8])
def test_batch_equals_single_frames(cuda_ctx, streams):
    import torch

    frames = _small_batch()
    _upload(cuda_ctx, frames)
    outs = _outputs(frames)
    b = gi.Batch(0)
    for f, o in zip(frames, outs):
        b.add_frame(f.scene, f.camera, f.lights, f.maps, f.params, o)
    b.build(streams)
    info = b.info()
    assert info["frames"] == len(frames) and info["streams"] == streams and info["kernel_launches"] > 0
    for _ in range(2):  # replays are idempotent
        outs_prev = [o.clone() for o in outs]
        b.run()
        torch.cuda.synchronize()
    for o, p in zip(outs, outs_prev):
        assert torch.equal(o, p)
    for f, o in zip(frames, outs):
        got = o.cpu().numpy()
        for l in range(len(f.lights)):
            ref, _ = _single(cuda_ctx, f, l)
            assert np.array_equal(got[l], ref), f"light {l} of a {f.triangles}-triangle scene differs"
    b.close()


@pytest.mark.gpu
def test_batch_one_light_matches_oracle(cuda_ctx):
    import torch

    frames = _small_batch(n=2)
    _upload(cuda_ctx, frames)
    outs = _outputs(frames)
    b = gi.Batch(0)
    for f, o in zip(frames, outs):
        b.add_frame(f.scene, f.camera, f.lights, f.maps, f.params, o)
    b.build(2)
    b.run()
    torch.cuda.synchronize()
    f = frames[1]
    l = len(f.lights) - 1
    fr = gi.frame_setup(f.lights[l], f.camera)
    p, n, i = f.scene.arrays()
    mp = f.maps[l]
    W, H = f.camera.width, f.camera.height
    d_ref = oracle.shadow_map(p, i, fr.light_mvp, mp.width, mp.height, mp.bias_mode, mp.constant_bias,
                              mp.offset_factor, mp.offset_units)
    pos, nrm = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    vis_ref = oracle.visibility(f.params.to_c(fr), d_ref, mp.width, mp.height, pos, nrm, W, H)
    assert np.array_equal(outs[1].cpu().numpy()[l], vis_ref.reshape(H, W))
    b.close()


@pytest.mark.gpu
def test_batch_autotune_keeps_results(cuda_ctx):
    import torch

    frames = _small_batch(n=4)
    _upload(cuda_ctx, frames)
    outs = _outputs(frames)
    b = gi.Batch(0)
    for f, o in zip(frames, outs):
        b.add_frame(f.scene, f.camera, f.lights, f.maps, f.params, o)
    b.build(4)
    b.run()
    torch.cuda.synchronize()
    first = [o.clone() for o in outs]
    for o in outs:
        o.fill_(-3.0)
    t = b.autotune(repeats=1)
    assert t["tiny_px"] < t["coop_px"] <= 1024 and t["streams"] >= 1 and t["best_ms"] > 0
    b.run()
    torch.cuda.synchronize()
    for o, p in zip(outs, first):
        assert torch.equal(o, p)
    b.close()


@pytest.mark.gpu
def test_batch_rejects_bad_input(cuda_ctx):
    frames = _small_batch(n=1)
    _upload(cuda_ctx, frames)
    f = frames[0]
    b = gi.Batch(0)
    with pytest.raises(gi.GIError):
        b.build(2)  # empty batch
    with pytest.raises(gi.GIError):
        b.run()  # not built
    import torch

    o = torch.zeros((len(f.lights), f.camera.height, f.camera.width), device="cuda")
    bad = [gi.MapParams(0, 0)] * len(f.lights)
    with pytest.raises(gi.GIError):
        b.add_frame(f.scene, f.camera, f.lights, bad, f.params, o)
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("tech", [api.GI_TECH_PCF, api.GI_TECH_PCSS_POISSON, api.GI_TECH_SMSR_NONCONSERVATIVE])
@pytest.mark.parametrize("tile", [(32, 4), (64, 8), (256, 16)])
def test_persistent_batch_equals_graph_batch(cuda_ctx, tech, tile):
    """One persistent visibility launch over every (light-frame, tile) item
    gives the graph mode's images bit for bit (which equal gi_render_frame)."""
    import torch

    frames = _small_batch(n=7, W=200, H=110)
    for f in frames:
        p = gi.ShadowParams.defaults(tech)
        p.light_radius = 0.5
        p.pcss_min_blocker_depth = 0.0
        p.kernel_order = 5
        f.params = p
    _upload(cuda_ctx, frames)
    graph_outs, pers_outs = _outputs(frames), _outputs(frames)
    bg, bp = gi.Batch(0), gi.Batch(0)
    for f, og, op in zip(frames, graph_outs, pers_outs):
        bg.add_frame(f.scene, f.camera, f.lights, f.maps, f.params, og)
        bp.add_frame(f.scene, f.camera, f.lights, f.maps, f.params, op)
    bg.build(3)
    bp.build_persistent(3, tile[0], tile[1])
    info = bp.info()
    n_lf = sum(len(f.lights) for f in frames)
    assert info["persistent"] and (info["tile_w"], info["tile_h"]) == tile
    assert info["work_items"] == n_lf * ((200 + tile[0] - 1) // tile[0]) * ((110 + tile[1] - 1) // tile[1])
    for _ in range(2):
        bg.run()
        bp.run()
    torch.cuda.synchronize()
    for og, op in zip(graph_outs, pers_outs):
        assert torch.equal(og.view(torch.int32), op.view(torch.int32))
    assert float((pers_outs[0] < 1.0).float().mean()) > 0.0
    bg.close()
    bp.close()


@pytest.mark.gpu
def test_persistent_autotune_and_rejections(cuda_ctx):
    import torch

    frames = _small_batch(n=3)
    _upload(cuda_ctx, frames)
    outs = _outputs(frames)
    b = gi.Batch(0)
    for f, o in zip(frames, outs):
        b.add_frame(f.scene, f.camera, f.lights, f.maps, f.params, o)
    b.build(2)
    b.run()
    torch.cuda.synchronize()
    ref = [o.clone() for o in outs]
    t = b.autotune_persistent(repeats=1)
    assert t["persistent"] and t["tile_w"] % 32 == 0 and t["work_items"] > 0 and t["best_ms"] > 0
    for o in outs:
        o.fill_(-3.0)
    b.run()
    torch.cuda.synchronize()
    for o, r in zip(outs, ref):
        assert torch.equal(o, r)
    with pytest.raises(gi.GIError):
        b.build_persistent(2, 48, 8)  # tile width not a multiple of 32
    b.close()
    # a moment technique needs per-light prepared maps: refused
    vsm = gi.Batch(0)
    f = frames[0]
    p = gi.ShadowParams.defaults(api.GI_TECH_VSM)
    cam = gi.ViewSpec(eye=f.camera.eye, at=f.camera.at, width=128, height=128)
    maps = [gi.MapParams(256, 256)] * len(f.lights)
    o = torch.zeros((len(f.lights), 128, 128), device="cuda")
    vsm.add_frame(f.scene, cam, f.lights, maps, p, o)
    with pytest.raises(gi.GIError):
        vsm.build_persistent(1, 64, 8)
    vsm.close()
