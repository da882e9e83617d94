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
