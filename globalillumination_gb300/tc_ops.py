"""Thin torch wrappers over the tcgen05 convolution kernels (gi_surrogate.h).

Tensors are NHWC CUDA tensors; BF16 tensors are torch.bfloat16 (same bits
as the C ABI's uint16 BF16).  Nothing here computes on its own: every
function is one C ABI call on the current stream, so the CUDA extension
must be loaded (there is no fallback).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _capi as api
from ._capi import check


def _lib():
    return api.load()


def _p(t) -> C.c_void_p:
    return C.c_void_p(int(t.data_ptr())) if t is not None else None


def _s() -> C.c_void_p:
    return C.c_void_p(int(torch.cuda.current_stream().cuda_stream))


def _need(t: torch.Tensor, numel: int, dtype, what: str) -> None:
    """Device tensors handed to the kernels must be CUDA, contiguous and large enough."""
    if not t.is_cuda or t.dtype != dtype or not t.is_contiguous() or t.numel() < numel:
        raise ValueError(f"{what}: need a contiguous CUDA {dtype} tensor of >= {numel} elements, "
                         f"got {t.dtype} {tuple(t.shape)} on {t.device}")


def nkb_pad(cin: int, ksize: int) -> int:
    nkb = ksize * ksize * cin // 8
    return (nkb + 3) // 4 * 4


def pack_weights(w: torch.Tensor, cin: int, flip: bool = False) -> torch.Tensor:
    """FP32 [cout, cin_real, k, k] -> packed BF16 ([cout or cin] x kblocks x 8)."""
    cout, cin_real, k, _ = w.shape
    kin = cout if flip else cin
    rows = cin if flip else cout
    out = torch.empty((rows, nkb_pad(kin, k), 8), dtype=torch.bfloat16, device=w.device)
    check(_lib().gi_pack_conv_weights(_p(w.contiguous()), cout, cin_real, cin, k, 1 if flip else 0, _p(out), _s()),
          "gi_pack_conv_weights")
    return out


def unpack_grad(dw_packed: torch.Tensor, cout: int, cin_real: int, cin: int, k: int) -> torch.Tensor:
    out = torch.empty((cout, cin_real, k, k), dtype=torch.float32, device=dw_packed.device)
    check(_lib().gi_unpack_conv_grad(_p(dw_packed), cout, cin_real, cin, k, _p(out), _s()), "gi_unpack_conv_grad")
    return out


def conv2d(x: torch.Tensor, wp: torch.Tensor, cout: int, ksize: int, bias: torch.Tensor | None = None,
           relu: bool = False, mask: torch.Tensor | None = None, out: torch.Tensor | None = None, out_off: int = 0,
           out32: torch.Tensor | None = None, err: torch.Tensor | None = None) -> torch.Tensor:
    """NHWC BF16 convolution (stride 1, zero padding) on the tensor cores."""
    n, h, w, cin = x.shape
    if out is None and out32 is None:
        out = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device=x.device)
    stride = out.shape[-1] if out is not None else cout
    _need(x, n * h * w * cin, torch.bfloat16, "x")
    _need(wp, wp.shape[0] * nkb_pad(cin, ksize) * 8, torch.bfloat16, "packed weights")
    if wp.shape[0] < cout:
        raise ValueError("packed weights have fewer rows than cout")
    if out is not None:
        _need(out, n * h * w * stride, torch.bfloat16, "out")
        if out_off + cout > stride:
            raise ValueError("out_off + cout exceeds the channels of out")
    if out32 is not None:
        _need(out32, n * h * w * cout, torch.float32, "out32")
    if mask is not None:
        _need(mask, n * h * w * stride, torch.bfloat16, "mask")
    if bias is not None:
        _need(bias, cout, torch.float32, "bias")
    check(_lib().gi_conv2d_bf16(_p(x), n, h, w, cin, _p(wp), _p(bias), cout, ksize,
                                api.GI_ACT_RELU if relu else api.GI_ACT_NONE, _p(mask), _p(out), stride, out_off,
                                _p(out32), _p(err), _s()), "gi_conv2d_bf16")
    return out if out is not None else out32


def conv2d_fused(x: torch.Tensor, wp: torch.Tensor, cout: int, bias: torch.Tensor | None = None, relu: bool = True,
                 out: torch.Tensor | None = None, out_off: int = 0, pool: torch.Tensor | None = None,
                 upsample: bool = False, err: torch.Tensor | None = None) -> None:
    """3x3 convolution (cin % 16 == 0) with the max-pool and / or the 2x
    nearest upsampling of its output fused into the epilogue: `pool`
    ([n, h/2, w/2, cout]) receives maxpool2(output); with `upsample`, `out`
    is [n, 2h, 2w, C] and receives upsample2(output) at channel out_off."""
    n, h, w, cin = x.shape
    _need(x, n * h * w * cin, torch.bfloat16, "x")
    _need(wp, wp.shape[0] * nkb_pad(cin, 3) * 8, torch.bfloat16, "packed weights")
    stride = out.shape[-1] if out is not None else cout
    scale = 4 if upsample else 1
    if out is not None:
        _need(out, n * h * w * scale * stride, torch.bfloat16, "out")
        if out_off + cout > stride:
            raise ValueError("out_off + cout exceeds the channels of out")
    if pool is not None:
        _need(pool, n * (h // 2) * (w // 2) * cout, torch.bfloat16, "pool")
    if bias is not None:
        _need(bias, cout, torch.float32, "bias")
    check(_lib().gi_conv2d_fused_bf16(_p(x), n, h, w, cin, _p(wp), _p(bias), cout,
                                      api.GI_ACT_RELU if relu else api.GI_ACT_NONE, _p(out), stride, out_off,
                                      _p(pool), 1 if upsample else 0, _p(err), _s()), "gi_conv2d_fused_bf16")


def conv2d_head(x: torch.Tensor, wp: torch.Tensor, cout: int, bias: torch.Tensor, head_w: torch.Tensor,
                head_b: torch.Tensor, out: torch.Tensor, relu: bool = True, err: torch.Tensor | None = None):
    """3x3 convolution with a fused two-output 1x1 head: out (FP32, [.., 2]) only."""
    n, h, w, cin = x.shape
    _need(x, n * h * w * cin, torch.bfloat16, "x")
    _need(out, n * h * w * 2, torch.float32, "out")
    _need(head_w, 2 * cout, torch.float32, "head_w")
    _need(head_b, 2, torch.float32, "head_b")
    _need(bias, cout, torch.float32, "bias")
    check(_lib().gi_conv2d_head_bf16(_p(x), n, h, w, cin, _p(wp), _p(bias), cout,
                                     api.GI_ACT_RELU if relu else api.GI_ACT_NONE, _p(head_w), _p(head_b), _p(out),
                                     _p(err), _s()), "gi_conv2d_head_bf16")
    return out


def conv2d_wgrad(x: torch.Tensor, dy: torch.Tensor, cout: int, ksize: int, dw: torch.Tensor,
                 db: torch.Tensor | None = None, scratch: torch.Tensor | None = None,
                 err: torch.Tensor | None = None) -> torch.Tensor:
    """dw (FP32, packed layout) += weight gradient; db += bias gradient."""
    n, h, w, cin = x.shape
    _need(x, n * h * w * cin, torch.bfloat16, "x")
    _need(dy, n * h * w * cout, torch.bfloat16, "dy")
    _need(dw, cout * nkb_pad(cin, ksize) * 8, torch.float32, "dw")
    if db is not None:
        _need(db, cout, torch.float32, "db")
    need = int(_lib().gi_conv2d_wgrad_scratch_floats(n, h, w, cin, cout, ksize))
    if scratch is None or scratch.numel() < need:
        scratch = torch.empty(need, dtype=torch.float32, device=x.device)
    check(_lib().gi_conv2d_wgrad_bf16(_p(x), _p(dy), n, h, w, cin, cout, ksize, _p(dw), _p(db), _p(scratch), _p(err),
                                      _s()), "gi_conv2d_wgrad_bf16")
    return scratch


def set_wait_limit(polls: int) -> None:
    """Polls per mbarrier wait in the tcgen05 kernels (default 2^20)."""
    check(_lib().gi_tc_set_wait_limit(int(polls)), "gi_tc_set_wait_limit")


def wait_limit() -> int:
    return int(_lib().gi_tc_wait_limit())


def set_test_withhold(enable: bool) -> None:
    """Test switch: the kernels withhold their first asynchronous stage, so a wait runs out."""
    check(_lib().gi_tc_set_test_withhold(1 if enable else 0), "gi_tc_set_test_withhold")


def maxpool2(x: torch.Tensor) -> torch.Tensor:
    n, h, w, c = x.shape
    y = torch.empty((n, h // 2, w // 2, c), dtype=x.dtype, device=x.device)
    check(_lib().gi_maxpool2_bf16(_p(x), n, h, w, c, _p(y), _s()), "gi_maxpool2_bf16")
    return y


def maxpool2_bwd(x: torch.Tensor, y: torch.Tensor, dy: torch.Tensor) -> torch.Tensor:
    n, h, w, c = x.shape
    dx = torch.empty_like(x)
    check(_lib().gi_maxpool2_bwd_bf16(_p(x), _p(y), _p(dy), n, h, w, c, _p(dx), _s()), "gi_maxpool2_bwd_bf16")
    return dx


def upsample2(x: torch.Tensor, out: torch.Tensor, out_off: int = 0) -> torch.Tensor:
    n, h, w, c = x.shape
    check(_lib().gi_upsample2_bf16(_p(x), n, h, w, c, _p(out), out.shape[-1], out_off, _s()), "gi_upsample2_bf16")
    return out


def upsample2_bwd(dy: torch.Tensor, c: int, off: int = 0) -> torch.Tensor:
    n, H, W, cs = dy.shape
    dx = torch.empty((n, H // 2, W // 2, c), dtype=dy.dtype, device=dy.device)
    check(_lib().gi_upsample2_bwd_bf16(_p(dy), n, H // 2, W // 2, c, cs, off, _p(dx), _s()), "gi_upsample2_bwd_bf16")
    return dx


def channel_slice(x: torch.Tensor, off: int, c: int) -> torch.Tensor:
    pixels = x.numel() // x.shape[-1]
    y = torch.empty(x.shape[:-1] + (c,), dtype=x.dtype, device=x.device)
    check(_lib().gi_channel_slice_bf16(_p(x), pixels, x.shape[-1], off, c, _p(y), _s()), "gi_channel_slice_bf16")
    return y


def channel_slice_add(x: torch.Tensor, y: torch.Tensor, off: int) -> torch.Tensor:
    pixels = x.numel() // x.shape[-1]
    check(_lib().gi_channel_slice_add_bf16(_p(x), pixels, x.shape[-1], _p(y), y.shape[-1], off, _s()),
          "gi_channel_slice_add_bf16")
    return y


def adam(p: torch.Tensor, g: torch.Tensor, m: torch.Tensor, v: torch.Tensor, lr: float, step: int,
         beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, grad_scale: float = 1.0) -> None:
    check(_lib().gi_adam_f32(_p(p), _p(g), _p(m), _p(v), p.numel(), lr, beta1, beta2, eps, step, grad_scale, _s()),
          "gi_adam_f32")
