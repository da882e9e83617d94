"""The light map's min-max pyramid and the exact tap skipping built on it.

Tap skipping tests small texel boxes (up to 3 x 3) from the map itself and
larger ones from the pyramid when the context builds it; both settings are
run.

gi_light_map_minmax against numpy block minima / maxima on random maps and
on a rendered light map; and PCSS (Poisson) visibility that reads the
pyramid against the oracle, which runs every tap, bit for bit: on maps with
many fully lit and fully shadowed receivers, on a map whose shape gets no
pyramid, and through gi_visibility with a depth pointer that is not 16-byte
aligned (no pyramid either)."""
import numpy as np
import pytest

import globalillumination_gb300 as gi
import oracle
from globalillumination_gb300 import _capi as api, scenes

pytestmark = pytest.mark.gpu


def _np_levels(m):
    out = []
    H, W = m.shape
    for L in range(1, 7):
        b = m.reshape(H >> L, 1 << L, W >> L, 1 << L)
        out.append(np.stack([b.min(axis=(1, 3)), b.max(axis=(1, 3))], axis=-1))
    return out


@pytest.mark.parametrize("H,W", [(64, 64), (128, 320), (1024, 1024)])
def test_pyramid_equals_numpy_block_min_max(cuda_ctx, H, W):
    import torch

    rng = np.random.default_rng(H * 7 + W)
    m = rng.random((H, W), dtype=np.float32)
    m[rng.random((H, W)) < 0.3] = 1.0
    d = torch.from_numpy(m).cuda()
    got = gi.light_map_minmax(cuda_ctx, d, W, H)
    torch.cuda.synchronize()
    for L, (g, want) in enumerate(zip(got, _np_levels(m)), start=1):
        assert np.array_equal(g.cpu().numpy(), want), f"level {L}"


def test_pyramid_rejects_unsupported_shapes(cuda_ctx):
    import torch

    d = torch.zeros(100 * 64, device="cuda")
    with pytest.raises(gi.GIError):
        gi.light_map_minmax(cuda_ctx, d, 100, 64)


def _frame(spheres, S, W, H, radius):
    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=spheres)
    w.params.light_radius = radius
    return w


@pytest.mark.parametrize("S,spheres,radius", [(1024, 40, 0.25), (960, 40, 0.25), (2048, 64, 1.5)])
@pytest.mark.parametrize("pyramid", [False, True])
def test_pcss_with_pyramid_equals_oracle(cuda_ctx, S, spheres, radius, pyramid):
    import torch

    cuda_ctx.set_tap_pyramid(pyramid)
    W, H = 640, 360
    w = _frame(spheres, S, W, H, radius)
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, w.params, W, H, bufs, store_gbuffer=True)
    torch.cuda.synchronize()
    p, n, i = w.scene.arrays()
    d = bufs.depth.cpu().numpy()
    tab = np.concatenate([gi.poisson_table(16).reshape(-1), gi.poisson_table(32).reshape(-1)])
    pos, nrm = bufs.pos.cpu().numpy(), bufs.nrm.cpu().numpy()
    want = oracle.visibility(w.params.to_c(fr), d, S, S, pos, nrm, W, H, tab)
    got = bufs.vis.cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"{int((got != want).sum())} pixels differ"
    # the unfused pass, once from the same buffer and once from a copy at a
    # 4-byte offset (no pyramid), gives the same bits
    out = torch.empty_like(bufs.vis)
    gi.compute_visibility(cuda_ctx, w.params, fr, bufs.depth, S, S, bufs.pos, bufs.nrm, out, W, H)
    shifted = torch.empty(S * S + 1, device="cuda")
    shifted[1:].copy_(bufs.depth)
    out2 = torch.empty_like(bufs.vis)
    gi.compute_visibility(cuda_ctx, w.params, fr, shifted[1:], S, S, bufs.pos, bufs.nrm, out2, W, H)
    torch.cuda.synchronize()
    assert torch.equal(out.view(torch.int32), bufs.vis.view(torch.int32))
    assert torch.equal(out2.view(torch.int32), bufs.vis.view(torch.int32))
    lit = float((bufs.vis == 1.0).float().mean())
    assert 0.05 < lit < 0.99  # the frame has lit pixels to skip and others to filter
    cuda_ctx.set_tap_pyramid(False)


@pytest.mark.parametrize("pyramid", [False, True])
@pytest.mark.parametrize("order", [3, 5])
def test_pcf_tap_skipping_equals_oracle(cuda_ctx, pyramid, order):
    import torch

    cuda_ctx.set_tap_pyramid(pyramid)
    W, H, S = 512, 300, 1024
    w = scenes.hard_pcf_1024(width=W, height=H, map_size=S)
    w.params.kernel_order = order
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, w.params, W, H, bufs, store_gbuffer=True)
    torch.cuda.synchronize()
    want = oracle.visibility(w.params.to_c(fr), bufs.depth.cpu().numpy(), S, S, bufs.pos.cpu().numpy(),
                             bufs.nrm.cpu().numpy(), W, H)
    got = bufs.vis.cpu().numpy()
    cuda_ctx.set_tap_pyramid(False)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"{int((got != want).sum())} pixels differ"
    assert ((got > 0.25) & (got < 1.0)).sum() > 100
