"""Learned PCSS surrogate: a BF16 U-Net on the tcgen05 convolution kernels.

The network (4 levels, 32 / 64 / 96 / 128 channels, two 3x3 convolutions
per level on each side, 2x2 max pooling, nearest upsampling with skip
concatenation, a 1x1 head with 16 outputs of which 0 is the visibility and
1 the predicted absolute error) maps the per-pixel features of
gi_surrogate_features to the PCSS (Poisson) visibility of the frame.
gi_surrogate_finish clamps the prediction and recomputes the exact PCSS
value wherever the predicted error exceeds the threshold (0.02).

Forward, backward (data gradients as convolutions with flipped weights and
a ReLU-derivative mask, weight gradients with the tcgen05 weight-gradient
kernel), the loss and Adam all run on this library's kernels; torch only
owns the buffers.  The reference has no learned component (its soft
shadows are the PCSS shader, SoftShadowMapping/Shaders/SoftShadow/
PlausibleSoftShadow.frag:556-633).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _capi as api
from . import tc_ops as ops
from ._capi import check
from .shadow import Context, Frame, MapParams, Scene, ShadowParams, ViewSpec, frame_setup, _f16, _ptr

ERR_THRESHOLD = 0.02
FEATURES = 16  # channels of the feature tensor (4 used)
HEAD = 16     # channels of the head (0: visibility, 1: predicted error)


@dataclass
class Layer:
    name: str
    cin_real: int
    cin: int
    cout: int
    k: int
    w: torch.Tensor = None
    b: torch.Tensor = None
    m: list = field(default_factory=list)
    v: list = field(default_factory=list)
    wp: torch.Tensor = None
    wflip: torch.Tensor = None
    dwp: torch.Tensor = None
    db: torch.Tensor = None

    def flops_per_pixel(self) -> int:
        return 2 * self.k * self.k * self.cin_real * self.cout


# (name, cin_real, cin, cout, k)
ARCH = [
    ("e0a", 4, FEATURES, 32, 3), ("e0b", 32, 32, 32, 3),
    ("e1a", 32, 32, 64, 3), ("e1b", 64, 64, 64, 3),
    ("e2a", 64, 64, 96, 3), ("e2b", 96, 96, 96, 3),
    ("e3a", 96, 96, 128, 3), ("e3b", 128, 128, 128, 3),
    ("d2a", 224, 224, 96, 3), ("d2b", 96, 96, 96, 3),
    ("d1a", 160, 160, 64, 3), ("d1b", 64, 64, 64, 3),
    ("d0a", 96, 96, 32, 3), ("d0b", 32, 32, 32, 3),
    ("head", 32, 32, HEAD, 1),
]
LEVEL_SCALE = {"e0": 1, "e1": 2, "e2": 4, "e3": 8, "d2": 4, "d1": 2, "d0": 1, "he": 1}


class UNet:
    def __init__(self, device: int = 0, seed: int = 0):
        self.device = torch.device("cuda", device)
        g = torch.Generator().manual_seed(seed)
        self.layers: dict[str, Layer] = {}
        for name, cr, ci, co, k in ARCH:
            L = Layer(name, cr, ci, co, k)
            std = math.sqrt(2.0 / (cr * k * k)) if name != "head" else math.sqrt(1.0 / (cr * k * k))
            L.w = (torch.randn(co, cr, k, k, generator=g) * std).to(self.device)
            L.b = torch.zeros(co, device=self.device)
            if name == "head":
                L.b[0] = 0.9  # start near "lit"
            L.m = [torch.zeros_like(L.w), torch.zeros_like(L.b)]
            L.v = [torch.zeros_like(L.w), torch.zeros_like(L.b)]
            L.dwp = torch.zeros((co, ops.nkb_pad(ci, k), 8), device=self.device)
            L.db = torch.zeros(co, device=self.device)
            self.layers[name] = L
        self.step_count = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._scratch = None
        self.repack()

    # ---- parameters --------------------------------------------------------------
    def repack(self) -> None:
        for L in self.layers.values():
            L.wp = ops.pack_weights(L.w, L.cin)
            L.wflip = ops.pack_weights(L.w, L.cin, flip=True) if L.name != "e0a" else None

    def state(self) -> dict:
        out = {}
        for n, L in self.layers.items():
            out[n + ".w"] = L.w.cpu().numpy()
            out[n + ".b"] = L.b.cpu().numpy()
        return out

    def load_state(self, st: dict) -> None:
        for n, L in self.layers.items():
            L.w.copy_(torch.from_numpy(np.asarray(st[n + ".w"])))
            L.b.copy_(torch.from_numpy(np.asarray(st[n + ".b"])))
        self.repack()

    def save(self, path: str) -> None:
        np.savez(path, **self.state())

    def load(self, path: str) -> None:
        with np.load(path) as z:
            self.load_state({k: z[k] for k in z.files})

    def flops(self, h: int, w: int, n: int = 1) -> int:
        """Multiply-add FLOPs (2 per MAC) of one forward over n x h x w pixels."""
        total = 0
        for L in self.layers.values():
            s = LEVEL_SCALE[L.name[:2]]
            total += L.flops_per_pixel() * (h // s) * (w // s)
        return total * n

    # ---- forward / backward --------------------------------------------------------
    def _conv(self, name, x, relu=True, out=None, out_off=0, out32=None):
        L = self.layers[name]
        return ops.conv2d(x, L.wp, L.cout, L.k, bias=L.b, relu=relu, out=out, out_off=out_off, out32=out32,
                          err=self.err)

    def _conv_fused(self, name, x, out, out_off, pool=None, upsample=False):
        L = self.layers[name]
        ops.conv2d_fused(x, L.wp, L.cout, bias=L.b, relu=True, out=out, out_off=out_off, pool=pool,
                         upsample=upsample, err=self.err)

    def forward(self, feat: torch.Tensor, out32: torch.Tensor | None = None, keep: bool = False) -> torch.Tensor:
        n, H, W, _ = feat.shape
        assert H % 8 == 0 and W % 8 == 0, "the U-Net needs height and width divisible by 8"
        bf = dict(dtype=torch.bfloat16, device=feat.device)
        a = {"f": feat}
        a["t0"] = self._conv("e0a", feat)
        a["cat0"] = torch.empty((n, H, W, 96), **bf)
        self._conv("e0b", a["t0"], out=a["cat0"], out_off=0)
        a["s0"] = ops.channel_slice(a["cat0"], 0, 32)
        a["p0"] = ops.maxpool2(a["s0"])
        a["t1"] = self._conv("e1a", a["p0"])
        a["cat1"] = torch.empty((n, H // 2, W // 2, 160), **bf)
        self._conv("e1b", a["t1"], out=a["cat1"], out_off=0)
        a["s1"] = ops.channel_slice(a["cat1"], 0, 64)
        a["p1"] = ops.maxpool2(a["s1"])
        a["t2"] = self._conv("e2a", a["p1"])
        a["cat2"] = torch.empty((n, H // 4, W // 4, 224), **bf)
        self._conv("e2b", a["t2"], out=a["cat2"], out_off=0)
        a["s2"] = ops.channel_slice(a["cat2"], 0, 96)
        a["p2"] = ops.maxpool2(a["s2"])
        a["t3"] = self._conv("e3a", a["p2"])
        a["b3"] = self._conv("e3b", a["t3"])
        ops.upsample2(a["b3"], a["cat2"], 96)
        a["u2a"] = self._conv("d2a", a["cat2"])
        a["u2"] = self._conv("d2b", a["u2a"])
        ops.upsample2(a["u2"], a["cat1"], 64)
        a["u1a"] = self._conv("d1a", a["cat1"])
        a["u1"] = self._conv("d1b", a["u1a"])
        ops.upsample2(a["u1"], a["cat0"], 32)
        a["u0a"] = self._conv("d0a", a["cat0"])
        a["u0"] = self._conv("d0b", a["u0a"])
        if out32 is None:
            out32 = torch.empty((n, H, W, HEAD), dtype=torch.float32, device=feat.device)
        self._conv("head", a["u0"], relu=False, out32=out32)
        self._acts = a if keep else None
        return out32

    def forward_fused(self, feat: torch.Tensor, head2: torch.Tensor) -> torch.Tensor:
        """Inference: forward with the 1x1 head fused into the last 3x3
        convolution's epilogue; head2 (FP32, [n, H, W, 2]) receives the
        visibility and the predicted error, the last activation is never
        stored.  The max-pools and upsamplings run in the epilogues of the
        convolutions that produce their inputs (gi_conv2d_fused_bf16), so
        the pooled and concatenated tensors are the same bits as forward()'s
        without its slice, pool and upsample passes."""
        n, H, W, _ = feat.shape
        assert H % 8 == 0 and W % 8 == 0, "the U-Net needs height and width divisible by 8"
        if getattr(self, "_hw_ver", -1) != self.step_count or not hasattr(self, "_hw"):
            L = self.layers["head"]
            self._hw = L.w[:2, :, 0, 0].to(torch.bfloat16).float().contiguous()
            self._hb = L.b[:2].contiguous()
            self._hw_ver = self.step_count
        bf = dict(dtype=torch.bfloat16, device=feat.device)
        # the encoders' 3x3 convolutions also write their pooled output, the
        # decoders' second convolutions write upsampled into the next
        # level's concatenation buffer (both fused into the epilogue)
        fused = self._conv_fused
        t0 = self._conv("e0a", feat)
        cat0 = torch.empty((n, H, W, 96), **bf)
        p0 = torch.empty((n, H // 2, W // 2, 32), **bf)
        fused("e0b", t0, cat0, 0, pool=p0)
        t1 = self._conv("e1a", p0)
        cat1 = torch.empty((n, H // 2, W // 2, 160), **bf)
        p1 = torch.empty((n, H // 4, W // 4, 64), **bf)
        fused("e1b", t1, cat1, 0, pool=p1)
        t2 = self._conv("e2a", p1)
        cat2 = torch.empty((n, H // 4, W // 4, 224), **bf)
        p2 = torch.empty((n, H // 8, W // 8, 96), **bf)
        fused("e2b", t2, cat2, 0, pool=p2)
        fused("e3b", self._conv("e3a", p2), cat2, 96, upsample=True)
        fused("d2b", self._conv("d2a", cat2), cat1, 64, upsample=True)
        fused("d1b", self._conv("d1a", cat1), cat0, 32, upsample=True)
        u0a = self._conv("d0a", cat0)
        L = self.layers["d0b"]
        ops.conv2d_head(u0a, L.wp, L.cout, L.b, self._hw, self._hb, head2, relu=True, err=self.err)
        return head2

    def _wgrad(self, name, x, dy):
        L = self.layers[name]
        self._scratch = ops.conv2d_wgrad(x, dy, L.cout, L.k, L.dwp, L.db, self._scratch, err=self.err)

    def _dgrad(self, name, dy, mask):
        L = self.layers[name]
        return ops.conv2d(dy, L.wflip, L.cin, L.k, mask=mask, err=self.err)

    def backward(self, dhead: torch.Tensor) -> None:
        a = self._acts
        assert a is not None, "forward(keep=True) first"
        for L in self.layers.values():
            L.dwp.zero_()
            L.db.zero_()
        self._wgrad("head", a["u0"], dhead)
        d = self._dgrad("head", dhead, a["u0"])
        self._wgrad("d0b", a["u0a"], d)
        d = self._dgrad("d0b", d, a["u0a"])
        self._wgrad("d0a", a["cat0"], d)
        dcat0 = self._dgrad("d0a", d, a["cat0"])
        d = ops.upsample2_bwd(dcat0, 64, 32)
        self._wgrad("d1b", a["u1a"], d)
        d = self._dgrad("d1b", d, a["u1a"])
        self._wgrad("d1a", a["cat1"], d)
        dcat1 = self._dgrad("d1a", d, a["cat1"])
        d = ops.upsample2_bwd(dcat1, 96, 64)
        self._wgrad("d2b", a["u2a"], d)
        d = self._dgrad("d2b", d, a["u2a"])
        self._wgrad("d2a", a["cat2"], d)
        dcat2 = self._dgrad("d2a", d, a["cat2"])
        d = ops.upsample2_bwd(dcat2, 128, 96)
        self._wgrad("e3b", a["t3"], d)
        d = self._dgrad("e3b", d, a["t3"])
        self._wgrad("e3a", a["p2"], d)
        d = self._dgrad("e3a", d, a["p2"])
        ops.channel_slice_add(ops.maxpool2_bwd(a["s2"], a["p2"], d), dcat2, 0)
        d = ops.channel_slice(dcat2, 0, 96)
        self._wgrad("e2b", a["t2"], d)
        d = self._dgrad("e2b", d, a["t2"])
        self._wgrad("e2a", a["p1"], d)
        d = self._dgrad("e2a", d, a["p1"])
        ops.channel_slice_add(ops.maxpool2_bwd(a["s1"], a["p1"], d), dcat1, 0)
        d = ops.channel_slice(dcat1, 0, 64)
        self._wgrad("e1b", a["t1"], d)
        d = self._dgrad("e1b", d, a["t1"])
        self._wgrad("e1a", a["p0"], d)
        d = self._dgrad("e1a", d, a["p0"])
        ops.channel_slice_add(ops.maxpool2_bwd(a["s0"], a["p0"], d), dcat0, 0)
        d = ops.channel_slice(dcat0, 0, 32)
        self._wgrad("e0b", a["t0"], d)
        d = self._dgrad("e0b", d, a["t0"])
        self._wgrad("e0a", a["f"], d)

    def adam_step(self, lr: float = 1e-3) -> None:
        self.step_count += 1
        for L in self.layers.values():
            g = ops.unpack_grad(L.dwp, L.cout, L.cin_real, L.cin, L.k)
            ops.adam(L.w, g, L.m[0], L.v[0], lr, self.step_count)
            ops.adam(L.b, L.db, L.m[1], L.v[1], lr, self.step_count)
        self.repack()

    def kernel_error(self) -> int:
        return int(self.err.item())


# ---- frames ------------------------------------------------------------------------
def features(ctx: Context, scene: Scene, frame: Frame, mp: MapParams, params: ShadowParams, W: int, H: int,
             depth: torch.Tensor, feat: torch.Tensor, stream=None) -> torch.Tensor:
    c = mp.to_c()
    p = params.to_c(frame)
    s = C.c_void_p(int((stream or torch.cuda.current_stream()).cuda_stream))
    check(api.load().gi_surrogate_features(ctx.handle, scene.handle, C.byref(c), _f16(frame.light_mvp),
                                           _f16(frame.camera_mvp), C.byref(p), W, H, _ptr(depth), _ptr(feat), s),
          "gi_surrogate_features")
    return feat


def finish(ctx: Context, scene: Scene, frame: Frame, mp: MapParams, params: ShadowParams, W: int, H: int,
           depth: torch.Tensor, head: torch.Tensor, feat: torch.Tensor, vis: torch.Tensor,
           fallback: torch.Tensor | None = None, threshold: float = ERR_THRESHOLD, stream=None) -> torch.Tensor:
    p = params.to_c(frame)
    s = C.c_void_p(int((stream or torch.cuda.current_stream()).cuda_stream))
    check(api.load().gi_surrogate_finish(ctx.handle, scene.handle, mp.width, mp.height, _ptr(depth),
                                         _f16(frame.camera_mvp), C.byref(p), W, H, _ptr(head), head.shape[-1],
                                         _ptr(feat),
                                         float(threshold), _ptr(vis), _ptr(fallback) if fallback is not None else None,
                                         s), "gi_surrogate_finish")
    return vis


def loss(head: torch.Tensor, target: torch.Tensor, feat: torch.Tensor, dhead: torch.Tensor, sums: torch.Tensor,
         err_weight: float = 0.5) -> None:
    """L1 loss of the visibility head plus the error head; writes dhead and adds the fixed-point
    totals to sums (int64 [3], see loss_totals)."""
    assert sums.dtype == torch.int64 and sums.numel() >= 3
    pixels = target.numel()
    check(api.load().gi_surrogate_loss(_ptr(head), _ptr(target), _ptr(feat), pixels, float(err_weight), _ptr(dhead),
                                       _ptr(sums), C.c_void_p(int(torch.cuda.current_stream().cuda_stream))),
          "gi_surrogate_loss")


def loss_totals(sums: torch.Tensor) -> np.ndarray:
    """(sum |v - t|, pixel count, sum error-head loss) as float64 from the fixed-point sums."""
    s = sums.cpu().numpy().astype(np.float64)
    return np.array([s[0] / 2.0 ** 32, s[1], s[2] / 2.0 ** 32])


class SurrogateFrame:
    """Preallocated buffers for surrogate frames of one size."""

    def __init__(self, net: UNet, map_size: int, W: int, H: int):
        dev = net.device
        self.net = net
        self.W, self.H = W, H
        self.depth = torch.empty(map_size * map_size, dtype=torch.float32, device=dev)
        self.feat = torch.empty((1, H, W, FEATURES), dtype=torch.bfloat16, device=dev)
        self.head = torch.empty((1, H, W, 2), dtype=torch.float32, device=dev)
        self.vis = torch.empty(W * H, dtype=torch.float32, device=dev)
        self.fallback = torch.zeros(1, dtype=torch.int32, device=dev)

    def render(self, ctx: Context, scene: Scene, frame: Frame, mp: MapParams, params: ShadowParams,
               threshold: float = ERR_THRESHOLD) -> torch.Tensor:
        features(ctx, scene, frame, mp, params, self.W, self.H, self.depth, self.feat)
        self.net.forward_fused(self.feat, self.head)
        finish(ctx, scene, frame, mp, params, self.W, self.H, self.depth, self.head, self.feat, self.vis,
               self.fallback, threshold)
        return self.vis


# ---- training data ---------------------------------------------------------------------
def training_scene(rng: np.random.Generator, seed: int):
    """A random training scene: mostly pcss_1080p-style sphere fields under an overhead light, a
    share of displaced spheres under oblique lights, 2048^2 or 4096^2 maps, 1080p or 2160p views
    (the features measure penumbrae in map texels and screen pixels, so both resolutions are seen)."""
    s = Scene()
    s.ground(10.0, 0.0)
    if rng.random() < 0.3:
        grid = int(rng.choice([128, 256, 384]))
        centre = (float(rng.uniform(-3.0, 3.0)), float(rng.uniform(1.8, 3.0)), float(rng.uniform(-3.0, 3.0)))
        s.displaced_sphere(grid, grid, float(rng.uniform(1.0, 2.2)), float(rng.uniform(0.1, 0.4)), centre,
                           seed ^ 0x2F5A3C1)
    else:
        spheres = int(rng.integers(16, 96))
        s.icosphere_field(spheres, 3, (-8.0, 0.2, -8.0), (8.0, 3.0, 8.0), 0.2, 1.0, seed)
    side = 4096 if rng.random() < 0.3 else 2048
    if rng.random() < 0.3:
        a = rng.uniform(0, 2 * math.pi)
        rr = rng.uniform(5.0, 9.0)
        eye = (float(rr * math.cos(a)), float(rng.uniform(6.0, 10.0)), float(rr * math.sin(a)))
    else:
        lx, lz = rng.uniform(-3.0, 3.0, 2)
        eye = (float(lx), float(rng.uniform(10.0, 14.0)), float(lz))
    light = ViewSpec(eye=eye, at=(0.0, 0.0, 0.0), width=side, height=side, fovy_deg=90.0)
    az = rng.uniform(0, 2 * math.pi)
    r = rng.uniform(14.0, 24.0)
    W, H = (3840, 2160) if rng.random() < 0.25 else (1920, 1080)
    camera = ViewSpec(eye=(float(r * math.sin(az)), float(rng.uniform(8.0, 16.0)), float(-r * math.cos(az))),
                      at=(0.0, 0.0, 0.0), width=W, height=H)
    mp = MapParams(side, side, bias_mode=api.GI_BIAS_POLYGON_OFFSET, offset_factor=4.0, offset_units=20.0)
    p = ShadowParams.defaults(api.GI_TECH_PCSS_POISSON)
    p.light_radius = float(rng.uniform(0.1, 0.5))
    p.pcss_min_blocker_depth = 0.0
    return s, light, camera, mp, p


# ---- checkpoints ---------------------------------------------------------------------
CHECKPOINT_VERSION = 1


def pack_checkpoint(net_state: dict, trainer_state: dict) -> dict:
    """Flat numpy archive of a training run: every layer's FP32 master
    weights and biases, their Adam moments, the optimiser step, and the
    trainer's position (next step, data RNG state, hyperparameters)."""
    import json

    out = {k: np.asarray(v) for k, v in net_state.items()}
    out["trainer_json"] = np.array(json.dumps(trainer_state))
    out["checkpoint_version"] = np.array(CHECKPOINT_VERSION)
    return out


def unpack_checkpoint(z) -> tuple[dict, dict]:
    import json

    if int(z["checkpoint_version"]) != CHECKPOINT_VERSION:
        raise ValueError("unsupported checkpoint version")
    net_state = {k: np.asarray(z[k]) for k in z.keys() if k not in ("trainer_json", "checkpoint_version")}
    return net_state, json.loads(str(z["trainer_json"]))


def net_full_state(net: "UNet") -> dict:
    out = {"step_count": np.array(net.step_count, np.int64)}
    for n, L in net.layers.items():
        out[n + ".w"] = L.w.cpu().numpy()
        out[n + ".b"] = L.b.cpu().numpy()
        out[n + ".mw"], out[n + ".mb"] = L.m[0].cpu().numpy(), L.m[1].cpu().numpy()
        out[n + ".vw"], out[n + ".vb"] = L.v[0].cpu().numpy(), L.v[1].cpu().numpy()
    return out


def load_net_full_state(net: "UNet", st: dict) -> None:
    for n, L in net.layers.items():
        for t, key in ((L.w, ".w"), (L.b, ".b"), (L.m[0], ".mw"), (L.m[1], ".mb"), (L.v[0], ".vw"), (L.v[1], ".vb")):
            t.copy_(torch.from_numpy(np.asarray(st[n + key])))
    net.step_count = int(st["step_count"])
    net.repack()


class Trainer:
    """Adam on random crops of freshly rendered PCSS frames; one crop per frame.

    The run is resumable: `save(path)` writes the weights, biases, Adam
    moments and step of every layer, the next step index and the data RNG's
    state; a new Trainer over a fresh UNet that `load`s it continues with the
    same crops and, the gradient reductions running in a fixed order, the
    same losses and weights bit for bit."""

    def __init__(self, ctx: Context, net: "UNet", batch: int = 16, crop: int = 256, lr: float = 1e-3,
                 scenes_in_pool: int = 24, seed: int = 0x5EED0003):
        self.ctx, self.net = ctx, net
        self.batch, self.crop, self.lr = batch, crop, lr
        self.scenes_in_pool, self.seed = scenes_in_pool, seed
        self.rng = np.random.default_rng(seed)
        self.pool = []
        for k in range(scenes_in_pool):
            s, light, camera, mp, p = training_scene(self.rng, seed + k)
            s.upload(ctx)
            self.pool.append((s, light, camera, mp, p))
        self.step = 0
        dev = net.device
        self._frames = {}  # (map side, W, H) -> (frame buffers, features, depth scratch)
        self.bfeat = torch.empty((batch, crop, crop, FEATURES), dtype=torch.bfloat16, device=dev)
        self.btarget = torch.empty((batch, crop, crop), dtype=torch.float32, device=dev)
        self.head = torch.empty((batch, crop, crop, HEAD), dtype=torch.float32, device=dev)
        self.dhead = torch.empty((batch, crop, crop, HEAD), dtype=torch.bfloat16, device=dev)
        self.sums = torch.zeros(3, dtype=torch.int64, device=dev)  # fixed point, see loss()

    def _buffers(self, side, W, H):
        from .shadow import allocate_frame

        if (side, W, H) not in self._frames:
            dev = self.net.device
            self._frames[(side, W, H)] = (allocate_frame(side, side, W, H),
                                          torch.empty((1, H, W, FEATURES), dtype=torch.bfloat16, device=dev),
                                          torch.empty(side * side, dtype=torch.float32, device=dev))
        return self._frames[(side, W, H)]

    def run(self, steps: int, log_every: int = 100, verbose: bool = True) -> list:
        """Runs `steps` optimiser steps; returns [{step, mae, err_l1, seconds}] every log_every steps and at the end."""
        from .shadow import render_frame

        rng, net, ctx = self.rng, self.net, self.ctx
        hist = []
        t0 = time.perf_counter()
        last = self.step + steps
        while self.step < last:
            for b in range(self.batch):
                s, light, camera, mp, p = self.pool[int(rng.integers(len(self.pool)))]
                # jitter the light within the scene's neighbourhood
                le = tuple(float(x) for x in np.asarray(light.eye) + rng.uniform(-1.0, 1.0, 3))
                lv = ViewSpec(eye=le, at=light.at, width=light.width, height=light.height, fovy_deg=light.fovy_deg)
                fr = frame_setup(lv, camera)
                W, H = camera.width, camera.height
                bufs, feat, depth2 = self._buffers(mp.width, W, H)
                render_frame(ctx, s, fr, mp, p, W, H, bufs)
                features(ctx, s, fr, mp, p, W, H, depth2, feat)
                y0 = int(rng.integers(0, H - self.crop + 1))
                x0 = int(rng.integers(0, W - self.crop + 1))
                self.bfeat[b].copy_(feat[0, y0:y0 + self.crop, x0:x0 + self.crop])
                self.btarget[b].copy_(bufs.vis.view(H, W)[y0:y0 + self.crop, x0:x0 + self.crop])
            net.forward(self.bfeat, out32=self.head, keep=True)
            self.sums.zero_()
            loss(self.head, self.btarget, self.bfeat, self.dhead, self.sums)
            net.backward(self.dhead)
            net.adam_step(self.lr)
            self.step += 1
            if self.step % log_every == 0 or self.step == last:
                s_ = loss_totals(self.sums)
                hist.append({"step": self.step, "mae": float(s_[0] / max(s_[1], 1.0)),
                             "err_l1": float(s_[2] / max(s_[1], 1.0)), "seconds": time.perf_counter() - t0})
                if verbose:
                    print(f"step {self.step} mae {hist[-1]['mae']:.5f} err-head {hist[-1]['err_l1']:.5f} "
                          f"{hist[-1]['seconds']:.1f}s", flush=True)
        if net.kernel_error():
            raise RuntimeError("a tcgen05 kernel reported a timed-out wait during training")
        return hist

    def state(self) -> dict:
        return {"step": self.step, "rng": self.rng.bit_generator.state, "batch": self.batch, "crop": self.crop,
                "lr": self.lr, "scenes_in_pool": self.scenes_in_pool, "seed": self.seed}

    def save(self, path: str) -> None:
        np.savez(path, **pack_checkpoint(net_full_state(self.net), self.state()))

    def load(self, path: str) -> None:
        with np.load(path) as z:
            net_state, st = unpack_checkpoint(z)
        for k in ("batch", "crop", "scenes_in_pool", "seed"):
            if st[k] != getattr(self, k):
                raise ValueError(f"checkpoint was made with {k} = {st[k]}, this trainer has {getattr(self, k)}")
        load_net_full_state(self.net, net_state)
        self.lr = st["lr"]
        self.step = int(st["step"])
        self.rng.bit_generator.state = st["rng"]


def train(ctx: Context, net: UNet, frames: int = 20000, batch: int = 16, crop: int = 256, lr: float = 1e-3,
          scenes_in_pool: int = 24, seed: int = 0x5EED0003, log_every: int = 100, verbose: bool = True) -> dict:
    """Adam on random crops of freshly rendered PCSS frames; one crop per frame (see Trainer)."""
    t0 = time.perf_counter()
    tr = Trainer(ctx, net, batch, crop, lr, scenes_in_pool, seed)
    steps = max(1, frames // batch)
    hist = tr.run(steps, log_every=log_every, verbose=verbose)
    return {"steps": steps, "frames": steps * batch, "batch": batch, "crop": crop, "history": hist,
            "seconds": time.perf_counter() - t0}
