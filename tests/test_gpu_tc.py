"""tcgen05 convolution kernels against a plain PyTorch FP32 reference.

Inputs are rounded to BF16 first; the reference convolves those values in
FP32 on the CPU.  Tolerances: the kernels accumulate in FP32 in another
order (|err| <= 1e-4 relative to the magnitude of the sum of |terms|), and
the BF16 outputs are additionally within one BF16 rounding (2^-8
relative) of the FP32 result."""
import pytest

torch = pytest.importorskip("torch")
import torch.nn.functional as F  # noqa: E402

from globalillumination_gb300 import tc_ops  # noqa: E402

pytestmark = pytest.mark.gpu


def _bf(t):
    return t.to(torch.bfloat16).to(torch.float32)


def _rand(*shape, seed=0):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(*shape, generator=g)


def _close(got, ref, absref, rtol=1e-4):
    err = (got - ref).abs()
    bound = rtol * absref + 1e-6
    assert bool((err <= bound).all()), f"max err {float(err.max())}, worst ratio {float((err / bound).max())}"


@pytest.mark.parametrize("P,K,N", [(300, 64, 48), (128, 16, 16), (1000, 200, 256), (77, 40, 96)])
def test_gemm_as_1x1_conv(P, K, N):
    A = _bf(_rand(P, K, seed=1))
    B = _bf(_rand(N, K, seed=2))
    x = A.reshape(1, 1, P, K).to(torch.bfloat16).cuda()
    wp = tc_ops.pack_weights(B.reshape(N, K, 1, 1).cuda(), K)
    y32 = torch.empty((P, N), device="cuda")
    tc_ops.conv2d(x, wp, N, 1, out32=y32)
    torch.cuda.synchronize()
    ref = A @ B.t()
    _close(y32.cpu(), ref, A.abs() @ B.abs().t())


@pytest.mark.parametrize("n,h,w,cin,cin_real,cout", [(2, 13, 17, 24, 24, 32), (1, 32, 40, 8, 4, 32),
                                                     (1, 9, 130, 96, 96, 64), (3, 16, 16, 160, 160, 128),
                                                     # slab kernel, taps stacked along N (cout 32 / 64), one
                                                     # stage (cin 16) and ragged row / column tiles
                                                     (2, 13, 131, 32, 32, 32), (1, 21, 40, 16, 16, 64),
                                                     (1, 3, 200, 16, 4, 32), (1, 19, 33, 64, 64, 64),
                                                     # slab kernel, not stacked: cout 16 and 48 (row stride
                                                     # wider than cout), cout 96 and 256
                                                     (1, 11, 20, 48, 48, 16), (1, 10, 150, 32, 32, 48),
                                                     (2, 7, 30, 32, 32, 96), (1, 5, 140, 16, 16, 256)])
def test_conv3x3_forward(n, h, w, cin, cin_real, cout):
    x = _bf(_rand(n, h, w, cin, seed=3))
    x[..., cin_real:] = 0
    wt = _bf(_rand(cout, cin_real, 3, 3, seed=4) * 0.2)
    b = _rand(cout, seed=5)
    xc = x.to(torch.bfloat16).cuda()
    wp = tc_ops.pack_weights(wt.cuda(), cin)
    y32 = torch.empty((n, h, w, cout), device="cuda")
    y = tc_ops.conv2d(xc, wp, cout, 3, bias=b.cuda(), relu=True, out32=y32,
                      out=torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda"))
    torch.cuda.synchronize()
    xn = x[..., :cin_real].permute(0, 3, 1, 2)
    ref = F.relu(F.conv2d(xn, wt, b, padding=1)).permute(0, 2, 3, 1)
    absref = F.conv2d(xn.abs(), wt.abs(), b.abs(), padding=1).permute(0, 2, 3, 1)
    _close(y32.cpu(), ref, absref)
    _close(y.float().cpu(), ref, absref + ref.abs() * 40.0)  # + one BF16 rounding


def test_conv_output_slice_and_mask():
    n, h, w, cin, cout = 1, 8, 8, 16, 32
    x = _bf(_rand(n, h, w, cin, seed=6)).to(torch.bfloat16).cuda()
    wp = tc_ops.pack_weights(_bf(_rand(cout, cin, 3, 3, seed=7)).cuda(), cin)
    full = torch.full((n, h, w, 64), 7.0, dtype=torch.bfloat16, device="cuda")
    mask = torch.zeros((n, h, w, 64), dtype=torch.bfloat16, device="cuda")
    mask[..., 32:48] = 1.0
    tc_ops.conv2d(x, wp, cout, 3, out=full, out_off=32, mask=mask)
    plain = tc_ops.conv2d(x, wp, cout, 3)
    torch.cuda.synchronize()
    assert bool((full[..., :32] == 7.0).all())
    assert torch.equal(full[..., 32:48], plain[..., :16])
    assert bool((full[..., 48:] == 0).all())


@pytest.mark.parametrize("n,h,w,cin,cout,pool,up", [(1, 16, 40, 32, 32, True, False),
                                                    (2, 10, 260, 64, 64, True, False),
                                                    (1, 6, 10, 96, 96, True, False),
                                                    (1, 8, 12, 128, 128, False, True),
                                                    (1, 9, 130, 96, 64, False, True),
                                                    (2, 14, 34, 16, 32, True, True)])
def test_conv_fused_pool_upsample_equal_separate_kernels(n, h, w, cin, cout, pool, up):
    """gi_conv2d_fused_bf16's pooled / upsampled outputs are bit-identical to
    gi_maxpool2_bf16 / gi_upsample2_bf16 of gi_conv2d_bf16's output, and
    channels outside the written slice stay untouched."""
    x = _bf(_rand(n, h, w, cin, seed=21)).to(torch.bfloat16).cuda()
    wp = tc_ops.pack_weights(_bf(_rand(cout, cin, 3, 3, seed=22) * 0.2).cuda(), cin)
    b = _rand(cout, seed=23).cuda()
    plain = tc_ops.conv2d(x, wp, cout, 3, bias=b, relu=True)
    C, off = cout + 16, 8
    scale = 2 if up else 1
    out = torch.full((n, h * scale, w * scale, C), 3.0, dtype=torch.bfloat16, device="cuda")
    pooled = torch.empty((n, h // 2, w // 2, cout), dtype=torch.bfloat16, device="cuda") if pool else None
    tc_ops.conv2d_fused(x, wp, cout, bias=b, relu=True, out=out, out_off=off, pool=pooled, upsample=up)
    torch.cuda.synchronize()
    if up:
        ref = torch.full_like(out, 3.0)
        tc_ops.upsample2(plain, ref, off)
        assert torch.equal(out, ref)
    else:
        assert torch.equal(out[..., off:off + cout], plain)
        assert bool((out[..., :off] == 3.0).all()) and bool((out[..., off + cout:] == 3.0).all())
    if pool:
        assert torch.equal(pooled, tc_ops.maxpool2(plain))


def test_conv_fused_rejects_bad_shapes():
    from globalillumination_gb300._capi import GIError

    x = torch.zeros((1, 5, 8, 32), dtype=torch.bfloat16, device="cuda")
    wp = tc_ops.pack_weights(torch.zeros(32, 32, 3, 3, device="cuda"), 32)
    with pytest.raises(GIError):  # odd height with pooling
        tc_ops.conv2d_fused(x, wp, 32, pool=torch.empty((1, 2, 4, 32), dtype=torch.bfloat16, device="cuda"))


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 12, 20, 32, 32), (1, 16, 24, 64, 96), (2, 8, 8, 96, 16),
                                            (1, 17, 140, 64, 32)])
def test_conv3x3_data_gradient(n, h, w, cin, cout):
    x = _bf(_rand(n, cin, h, w, seed=8)).requires_grad_(True)
    wt = _bf(_rand(cout, cin, 3, 3, seed=9) * 0.2)
    gy = _bf(_rand(n, cout, h, w, seed=10))
    F.conv2d(x, wt, padding=1).backward(gy)
    ref = x.grad.permute(0, 2, 3, 1)
    absref = torch.nn.grad.conv2d_input(x.shape, wt.abs(), gy.abs(), padding=1).permute(0, 2, 3, 1)
    wflip = tc_ops.pack_weights(wt.cuda(), cin, flip=True)
    dy = gy.permute(0, 2, 3, 1).contiguous().to(torch.bfloat16).cuda()
    dx32 = torch.empty((n, h, w, cin), device="cuda")
    tc_ops.conv2d(dy, wflip, cin, 3, out32=dx32)
    torch.cuda.synchronize()
    _close(dx32.cpu(), ref, absref)


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 12, 20, 32, 32), (1, 33, 47, 8, 32), (4, 16, 16, 64, 128),
                                            (1, 40, 64, 224, 96),
                                            # TMA kernel: 16- / 32- / 64-channel boxes, rows longer
                                            # than one 64-pixel chunk, several images, cout 256
                                            (1, 9, 70, 16, 32), (1, 10, 130, 96, 32), (1, 6, 65, 160, 64),
                                            (1, 5, 20, 32, 256), (3, 7, 9, 48, 16)])
def test_conv3x3_weight_gradient(n, h, w, cin, cout):
    x = _bf(_rand(n, cin, h, w, seed=11))
    wt = _bf(_rand(cout, cin, 3, 3, seed=12)).requires_grad_(True)
    b = torch.zeros(cout, requires_grad=True)
    gy = _bf(_rand(n, cout, h, w, seed=13))
    F.conv2d(x, wt, b, padding=1).backward(gy)
    absref = torch.nn.grad.conv2d_weight(x.abs(), wt.shape, gy.abs(), padding=1)
    xc = x.permute(0, 2, 3, 1).contiguous().to(torch.bfloat16).cuda()
    dy = gy.permute(0, 2, 3, 1).contiguous().to(torch.bfloat16).cuda()
    dwp = torch.zeros((cout, tc_ops.nkb_pad(cin, 3), 8), device="cuda")
    db = torch.zeros(cout, device="cuda")
    tc_ops.conv2d_wgrad(xc, dy, cout, 3, dwp, db)
    dw = tc_ops.unpack_grad(dwp, cout, cin, cin, 3)
    torch.cuda.synchronize()
    _close(dw.cpu(), wt.grad, absref)
    _close(db.cpu(), b.grad, gy.abs().sum((0, 2, 3)), rtol=1e-3)


@pytest.mark.parametrize("c", [16, 12])  # 16: the 8-channel kernels; 12: the per-element ones
def test_pool_upsample_helpers_bitwise(c):
    """The training helpers against a PyTorch restatement of their per-element
    rules (same operation order, BF16 rounding of FP32 results): max-pool,
    its gradient to the first maximum of each window, the upsampling
    gradient ((a + b) + c) + d, and the slice add."""
    g = torch.Generator().manual_seed(31)
    # coarse values so that windows hold ties
    x = (torch.randint(0, 6, (2, 8, 10, c), generator=g).float() * 0.25).to(torch.bfloat16).cuda()
    y = tc_ops.maxpool2(x)
    xf = x.float()
    win = torch.stack([xf[:, 0::2, 0::2], xf[:, 0::2, 1::2], xf[:, 1::2, 0::2], xf[:, 1::2, 1::2]])
    ref_y = torch.maximum(torch.maximum(torch.maximum(win[0], win[1]), win[2]), win[3]).to(torch.bfloat16)
    assert torch.equal(y, ref_y)
    dy = (torch.randn((2, 4, 5, c), generator=g)).to(torch.bfloat16).cuda()
    dx = tc_ops.maxpool2_bwd(x, y, dy)
    ref_dx = torch.zeros_like(xf)
    taken = torch.zeros_like(y.float(), dtype=torch.bool)
    for q, (oy, ox) in enumerate(((0, 0), (0, 1), (1, 0), (1, 1))):
        hit = (~taken) & (x[:, oy::2, ox::2] == y)
        ref_dx[:, oy::2, ox::2] = torch.where(hit, dy.float(), torch.zeros_like(dy.float()))
        taken |= hit
    assert torch.equal(dx.float(), ref_dx)
    stride, off = c + 16, 8
    up = (torch.randn((2, 8, 10, stride), generator=g)).to(torch.bfloat16).cuda()
    d = tc_ops.upsample2_bwd(up, c, off)
    uf = up.float()[..., off:off + c]
    ref_d = (((uf[:, 0::2, 0::2] + uf[:, 0::2, 1::2]) + uf[:, 1::2, 0::2]) + uf[:, 1::2, 1::2]).to(torch.bfloat16)
    assert torch.equal(d, ref_d)
    base = (torch.randn((2, 8, 10, stride), generator=g)).to(torch.bfloat16).cuda()
    add = (torch.randn((2, 8, 10, c), generator=g)).to(torch.bfloat16).cuda()
    ref_s = base.clone()
    ref_s[..., off:off + c] = (base.float()[..., off:off + c] + add.float()).to(torch.bfloat16)
    tc_ops.channel_slice_add(add, base, off)
    assert torch.equal(base, ref_s)


def test_pool_upsample_roundtrip():
    x = _bf(_rand(2, 8, 12, 16, seed=14)).to(torch.bfloat16).cuda()
    y = tc_ops.maxpool2(x)
    ref = F.max_pool2d(x.float().permute(0, 3, 1, 2), 2).permute(0, 2, 3, 1)
    assert torch.equal(y.float(), ref)
    up = torch.zeros((2, 8, 12, 32), dtype=torch.bfloat16, device="cuda")
    tc_ops.upsample2(y, up, 16)
    assert torch.equal(up[..., 16:].float(), F.interpolate(ref.permute(0, 3, 1, 2), scale_factor=2).permute(0, 2, 3, 1))
    d = tc_ops.upsample2_bwd(up, 16, 16)
    assert torch.equal(d.float(), 4 * y.float())
    dx = tc_ops.maxpool2_bwd(x, y, y)
    assert torch.equal(dx.float().sum(), y.float().sum())
