"""The learned PCSS surrogate: U-Net forward and gradients against a plain
PyTorch FP32 model with the same (BF16-rounded) weights, the frame entry
points (features / finish with exact fallback), and a short training run
that must reduce the loss."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.nn.functional as F  # noqa: E402

import globalillumination_gb300 as gi  # noqa: E402
from globalillumination_gb300 import _capi as api, scenes, surrogate as sg  # noqa: E402

pytestmark = pytest.mark.gpu


def _torch_unet(net, f):
    """FP32 reference of UNet.forward on NCHW input f (4 real channels)."""
    def conv(name, x, relu=True):
        L = net.layers[name]
        w = L.w.detach().cpu().to(torch.bfloat16).float()
        y = F.conv2d(x, w, L.b.detach().cpu(), padding=L.k // 2)
        return F.relu(y) if relu else y

    t0 = conv("e0a", f)
    s0 = conv("e0b", t0)
    t1 = conv("e1a", F.max_pool2d(s0, 2))
    s1 = conv("e1b", t1)
    t2 = conv("e2a", F.max_pool2d(s1, 2))
    s2 = conv("e2b", t2)
    t3 = conv("e3a", F.max_pool2d(s2, 2))
    b3 = conv("e3b", t3)
    u2 = conv("d2b", conv("d2a", torch.cat([s2, F.interpolate(b3, scale_factor=2)], 1)))
    u1 = conv("d1b", conv("d1a", torch.cat([s1, F.interpolate(u2, scale_factor=2)], 1)))
    u0 = conv("d0b", conv("d0a", torch.cat([s0, F.interpolate(u1, scale_factor=2)], 1)))
    return conv("head", u0, relu=False)


def _feat(n, H, W, seed=0):
    g = torch.Generator().manual_seed(seed)
    f = torch.zeros(n, H, W, sg.FEATURES)
    f[..., 0] = (torch.rand(n, H, W, generator=g) > 0.5).float() * 0.75 + 0.25
    f[..., 1] = torch.rand(n, H, W, generator=g) * 2 - 0.5
    f[..., 2] = torch.rand(n, H, W, generator=g) * 2
    f[..., 3] = 1.0
    return f.to(torch.bfloat16)


def test_unet_forward_matches_torch():
    net = sg.UNet(0, seed=3)
    f = _feat(2, 32, 48)
    out = net.forward(f.cuda())
    torch.cuda.synchronize()
    ref = _torch_unet(net, f.float()[..., :4].permute(0, 3, 1, 2)).permute(0, 2, 3, 1)
    got = out.cpu()
    rel = float((got - ref).norm() / ref.norm())
    assert rel < 2e-2, rel  # BF16 activations between layers
    assert net.kernel_error() == 0


def test_unet_gradients_match_torch():
    net = sg.UNet(0, seed=4)
    n, H, W = 2, 32, 32
    f = _feat(n, H, W, seed=1)
    g = torch.Generator().manual_seed(2)
    target = torch.rand(n, H, W, generator=g) * 0.75 + 0.25
    head = net.forward(f.cuda(), keep=True)
    dhead = torch.empty((n, H, W, sg.HEAD), dtype=torch.bfloat16, device="cuda")
    sums = torch.zeros(3, dtype=torch.int64, device="cuda")
    sg.loss(head, target.cuda(), f.cuda(), dhead, sums, err_weight=0.5)
    net.backward(dhead)
    torch.cuda.synchronize()
    # reference gradients with the same loss on the FP32 model
    params = {}
    for name, L in net.layers.items():
        params[name] = L.w.detach().cpu().to(torch.bfloat16).float().requires_grad_(True)

    def conv(name, x, relu=True):
        L = net.layers[name]
        y = F.conv2d(x, params[name], L.b.detach().cpu(), padding=L.k // 2)
        return F.relu(y) if relu else y

    x = f.float()[..., :4].permute(0, 3, 1, 2)
    t0 = conv("e0a", x)
    s0 = conv("e0b", t0)
    s1 = conv("e1b", conv("e1a", F.max_pool2d(s0, 2)))
    s2 = conv("e2b", conv("e2a", F.max_pool2d(s1, 2)))
    b3 = conv("e3b", conv("e3a", F.max_pool2d(s2, 2)))
    u2 = conv("d2b", conv("d2a", torch.cat([s2, F.interpolate(b3, scale_factor=2)], 1)))
    u1 = conv("d1b", conv("d1a", torch.cat([s1, F.interpolate(u2, scale_factor=2)], 1)))
    u0 = conv("d0b", conv("d0a", torch.cat([s0, F.interpolate(u1, scale_factor=2)], 1)))
    h = conv("head", u0, relu=False)
    v, e = h[:, 0], h[:, 1]
    P = n * H * W
    L = ((v - target).abs().sum() + 0.5 * (e - (v - target).abs().detach()).abs().sum()) / P
    L.backward()
    for name, Lr in net.layers.items():
        got = sg.ops.unpack_grad(Lr.dwp, Lr.cout, Lr.cin_real, Lr.cin, Lr.k).cpu()
        ref = params[name].grad
        cos = float(F.cosine_similarity(got.reshape(1, -1), ref.reshape(1, -1)))
        rel = float((got - ref).norm() / (ref.norm() + 1e-12))
        assert cos > 0.98 and rel < 0.2, (name, cos, rel)
    assert net.kernel_error() == 0


def test_fused_head_matches_separate_head():
    net = sg.UNet(0, seed=7)
    f = _feat(1, 40, 64, seed=3).cuda()
    full = net.forward(f)
    h2 = torch.empty((1, 40, 64, 2), device="cuda")
    net.forward_fused(f, h2)
    torch.cuda.synchronize()
    d = (full[..., :2] - h2).abs().max().item()
    assert d < 1e-3 * (1.0 + full[..., :2].abs().max().item()), d


def _pcss_frame(W=320, H=184, S=512):
    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=24)
    w.params.light_radius = 0.5
    return w


def test_surrogate_frame_fallback_is_exact(cuda_ctx):
    w = _pcss_frame()
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, w.params, W, H, bufs)
    net = sg.UNet(0, seed=5)
    sf = sg.SurrogateFrame(net, S, W, H)
    v_all = sf.render(cuda_ctx, w.scene, fr, w.map_params, w.params, threshold=-1.0).clone()
    n_fb = int(sf.fallback.item())
    torch.cuda.synchronize()
    ref = bufs.vis
    assert torch.equal(sf.depth.view(torch.int32), bufs.depth.view(torch.int32))
    assert torch.equal(v_all, ref)  # every pixel fell back to the exact PCSS
    feat = sf.feat.float().cpu().numpy()[0]
    assert n_fb == int((feat[..., 3] == 1.0).sum())
    # without fallback: background 0, failed pre-test = intensity, else clamped prediction
    sf.fallback.zero_()
    v_net = sf.render(cuda_ctx, w.scene, fr, w.map_params, w.params, threshold=math.inf).cpu().numpy().reshape(H, W)
    assert int(sf.fallback.item()) == 0
    I = w.params.shadow_intensity
    head = sf.head.cpu().numpy()[0]
    assert head.shape[-1] == 2
    m = feat[..., 3]
    assert (v_net[m == 0] == 0).all()
    assert (v_net[m == 0.5] == np.float32(I)).all()
    pred = np.clip(head[..., 0], I, 1.0)
    assert np.array_equal(v_net[m == 1], pred[m == 1].astype(np.float32))
    # hard-shadow feature equals the HARD technique on the same frame
    p_hard = gi.ShadowParams.defaults(api.GI_TECH_HARD)
    bufs2 = gi.allocate_frame(S, S, W, H)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, p_hard, W, H, bufs2)
    hard = bufs2.vis.cpu().numpy().reshape(H, W)
    assert np.array_equal(feat[..., 0], hard.astype(np.float32))


def test_short_training_reduces_loss(cuda_ctx):
    net = sg.UNet(0, seed=6)
    out = sg.train(cuda_ctx, net, frames=16 * 40, batch=16, crop=128, lr=1e-3, scenes_in_pool=4, log_every=10,
                   verbose=False)
    h = out["history"]
    assert h[-1]["mae"] < h[0]["mae"]
    assert net.kernel_error() == 0
