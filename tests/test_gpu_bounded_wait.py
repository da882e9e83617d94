"""Bounded mbarrier waits of the tcgen05 kernels: a wait that runs out ends the kernel cleanly.

With the test switch on, every convolution kernel withholds its first
asynchronous stage (the TMA loads of the persistent slab kernel and of the
3x3 weight-gradient kernel, the MMAs of the gather kernels), so its first
wait on that stage
can never complete.  With a short wait limit each kernel must then stop
issuing work, skip its tensor-memory reads, free its tensor memory, set bit
0 of the error word and return: the stream synchronises, and the next
normal call on the same context gives the right answer with a clear error
word.  No wait here is unbounded and nothing faults; the failure is a flag
that nothing sets.
"""
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


def _cases():
    """(name, run(err) -> result on the GPU, reference on the CPU, tolerance scale)."""
    out = []
    # persistent TMA slab kernel: 3x3, cin % 16 == 0
    x = _bf(_rand(1, 24, 200, 32, seed=11))
    wt = _bf(_rand(32, 32, 3, 3, seed=12) * 0.2)
    xc, wp = x.to(torch.bfloat16).cuda(), tc_ops.pack_weights(wt.cuda(), 32)

    def slab(err):
        y32 = torch.empty((1, 24, 200, 32), device="cuda")
        tc_ops.conv2d(xc, wp, 32, 3, out32=y32, err=err)
        return y32

    xn = x.permute(0, 3, 1, 2)
    out.append(("slab", slab, F.conv2d(xn, wt, padding=1).permute(0, 2, 3, 1),
                F.conv2d(xn.abs(), wt.abs(), padding=1).permute(0, 2, 3, 1)))
    # gather kernel: 1x1 convolution = GEMM
    A = _bf(_rand(300, 64, seed=13))
    B = _bf(_rand(48, 64, seed=14))
    Ac, Bp = A.reshape(1, 1, 300, 64).to(torch.bfloat16).cuda(), tc_ops.pack_weights(B.reshape(48, 64, 1, 1).cuda(), 64)

    def gemm(err):
        y32 = torch.empty((300, 48), device="cuda")
        tc_ops.conv2d(Ac, Bp, 48, 1, out32=y32, err=err)
        return y32

    out.append(("gather", gemm, A @ B.t(), A.abs() @ B.abs().t()))
    # weight gradient (1x1): dW[co, ci] = sum_p dy[p, co] x[p, ci]
    xg = _bf(_rand(1, 16, 16, 16, seed=15))
    dyg = _bf(_rand(1, 16, 16, 32, seed=16))
    xgc, dygc = xg.to(torch.bfloat16).cuda(), dyg.to(torch.bfloat16).cuda()

    def wgrad(err):
        dw = torch.zeros(32 * tc_ops.nkb_pad(16, 1) * 8, device="cuda")
        tc_ops.conv2d_wgrad(xgc, dygc, 32, 1, dw, err=err)
        return dw.reshape(32, -1)[:, :16]

    xf, df = xg.reshape(-1, 16), dyg.reshape(-1, 32)
    out.append(("wgrad", wgrad, df.t() @ xf, df.abs().t() @ xf.abs()))
    # weight gradient (3x3, TMA-fed kernel)
    x3 = _bf(_rand(1, 32, 6, 70, seed=17))
    d3 = _bf(_rand(1, 32, 6, 70, seed=18))
    x3c = x3.permute(0, 2, 3, 1).contiguous().to(torch.bfloat16).cuda()
    d3c = d3.permute(0, 2, 3, 1).contiguous().to(torch.bfloat16).cuda()

    def wgrad3(err):
        dw = torch.zeros(32 * tc_ops.nkb_pad(32, 3) * 8, device="cuda")
        tc_ops.conv2d_wgrad(x3c, d3c, 32, 3, dw, err=err)
        return tc_ops.unpack_grad(dw.reshape(32, -1, 8), 32, 32, 32, 3)

    ref3 = torch.nn.grad.conv2d_weight(x3, (32, 32, 3, 3), d3, padding=1)
    abs3 = torch.nn.grad.conv2d_weight(x3.abs(), (32, 32, 3, 3), d3.abs(), padding=1)
    out.append(("wgrad3x3", wgrad3, ref3, abs3))
    return out


def test_wait_that_runs_out_sets_error_and_context_recovers():
    default = tc_ops.wait_limit()
    cases = _cases()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    try:
        tc_ops.set_wait_limit(1 << 12)
        tc_ops.set_test_withhold(True)
        for name, run, _, _ in cases:
            err.zero_()
            run(err)
            torch.cuda.synchronize()  # the kernel returned
            assert int(err.item()) & 1, f"{name}: the withheld stage did not make a wait run out"
    finally:
        tc_ops.set_test_withhold(False)
        tc_ops.set_wait_limit(default)
    assert tc_ops.wait_limit() == default
    for name, run, ref, absref in cases:
        err.zero_()
        got = run(err).cpu()
        torch.cuda.synchronize()
        assert int(err.item()) == 0, f"{name}: error bit after recovery"
        bound = 1e-4 * absref + 1e-6
        assert bool(((got - ref).abs() <= bound).all()), f"{name}: wrong result after recovery"


def test_wait_limit_rejects_zero():
    from globalillumination_gb300._capi import GIError

    with pytest.raises(GIError):
        tc_ops.set_wait_limit(0)
