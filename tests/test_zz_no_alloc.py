"""gi_gbuffer_noalloc: the G-buffer pass for callers that cannot allocate.

Some callers cannot call cudaMalloc: a real-time frame loop in which
cudaMalloc's implicit device synchronisation would stall the frame, or an
application whose device memory is all owned by its own pool.  For them the
library has one allocation-free entry point, which keeps the pass's scratch
in a static device array (at most 1024 x 1024 pixels).  This test calls it
through the C ABI twice in a row, on two different scenes, and checks each
result against gi_gbuffer (bit for bit, the G-buffer tests' bar), so stale
scratch from the first call cannot leak into the second.  It also checks the
property the entry point exists for (a call leaves the device's free memory
unchanged) and a scene with more large triangles than the array's record
slots, whose surplus the pass rasterises in the setup threads.  It lives in
its own file, collected last, and creates its own context so it runs the
same alone or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api

pytestmark = pytest.mark.gpu


def _scene(kind):
    s = gi.Scene()
    s.ground(10.0, 0.0)
    if kind == 0:
        s.uv_sphere(48, 24, 1.0, (0.0, 1.2, 0.0))
        s.icosphere(2, 0.7, (2.0, 0.8, 1.0))
    else:
        s.icosphere_field(9, 2, (-6.0, 0.2, -6.0), (6.0, 2.5, 6.0), 0.3, 1.0, 0x5EED00AA)
    return s


def _noalloc(lib, d_pts, d_nrm, nv, d_idx, nt, mvp, W, H, pos, nrm, stream):
    return lib.gi_gbuffer_noalloc(C.c_void_p(d_pts.data_ptr()), C.c_void_p(d_nrm.data_ptr()), nv,
                                  C.c_void_p(d_idx.data_ptr()), nt, api.F16(*mvp.tolist()), W, H,
                                  C.c_void_p(pos.data_ptr()), C.c_void_p(nrm.data_ptr()),
                                  C.c_void_p(stream.cuda_stream))


def test_noalloc_gbuffer_matches_gbuffer_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = api.load()
    ctx = gi.Context(0)
    stream = torch.cuda.current_stream()
    cases = [(0, 512, 384, (0.0, 6.0, -9.0)), (1, 300, 170, (0.0, 11.0, -14.0))]
    for kind, W, H, eye in cases:
        s = _scene(kind)
        cam = gi.ViewSpec(eye=eye, at=(0.0, 0.5, 0.0), width=W, height=H)
        fr = gi.frame_setup(gi.ViewSpec(eye=(3, 9, 2), at=(0, 0, 0), width=64, height=64), cam)
        p, n, i = s.arrays()
        d_pts = torch.from_numpy(p.reshape(-1).copy()).cuda()
        d_nrm = torch.from_numpy(n.reshape(-1).copy()).cuda()
        d_idx = torch.from_numpy(i.reshape(-1).copy()).cuda()
        pos = torch.full((W * H * 4,), -7.0, dtype=torch.float32, device="cuda")
        nrm = torch.full((W * H * 4,), -7.0, dtype=torch.float32, device="cuda")
        st = _noalloc(lib, d_pts, d_nrm, p.shape[0], d_idx, i.shape[0], fr.camera_mvp, W, H, pos, nrm, stream)
        assert st == api.GI_OK, lib.gi_last_error_string()
        s.upload(ctx, stream)
        ref_pos = torch.empty_like(pos)
        ref_nrm = torch.empty_like(nrm)
        gi.render_gbuffer(ctx, s, fr.camera_mvp, W, H, ref_pos, ref_nrm, stream)
        torch.cuda.synchronize()
        a, b = pos.cpu().numpy(), ref_pos.cpu().numpy()
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"{int((a != b).sum())} position floats differ"
        a, b = nrm.cpu().numpy(), ref_nrm.cpu().numpy()
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"{int((a != b).sum())} normal floats differ"
        assert (b.reshape(-1, 4)[:, 3] == 1.0).sum() > 1000  # the scene is in view
    ctx.close()


def _gbuffer_pair(lib, ctx, s, mvp, W, H, stream):
    """Runs gi_gbuffer_noalloc and gi_gbuffer on scene `s`; returns both results."""
    import torch

    p, n, i = s.arrays()
    d_pts = torch.from_numpy(p.reshape(-1).copy()).cuda()
    d_nrm = torch.from_numpy(n.reshape(-1).copy()).cuda()
    d_idx = torch.from_numpy(i.reshape(-1).copy()).cuda()
    pos = torch.full((W * H * 4,), -7.0, dtype=torch.float32, device="cuda")
    nrm = torch.full((W * H * 4,), -7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    st = _noalloc(lib, d_pts, d_nrm, p.shape[0], d_idx, i.shape[0], mvp, W, H, pos, nrm, stream)
    assert st == api.GI_OK, lib.gi_last_error_string()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    s.upload(ctx, stream)
    ref_pos = torch.empty_like(pos)
    ref_nrm = torch.empty_like(nrm)
    gi.render_gbuffer(ctx, s, mvp, W, H, ref_pos, ref_nrm, stream)
    torch.cuda.synchronize()
    return free0, free1, (pos.cpu().numpy(), nrm.cpu().numpy()), (ref_pos.cpu().numpy(), ref_nrm.cpu().numpy())


def test_noalloc_gbuffer_allocates_nothing_and_spills_surplus_records():
    """20,000 triangles of at least 24 x 24 pixels each at 256 x 256, drawn with
    an identity camera matrix (vertices given in clip space): more than the
    16,384 record slots of the static array, so the surplus takes the
    in-thread path.  Both calls after the warm-up leave free memory as it was."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = api.load()
    ctx = gi.Context(0)
    stream = torch.cuda.current_stream()
    W = H = 256
    rng = np.random.default_rng(0x5EED0A11)
    T = 20000
    c = rng.uniform(-0.8, 0.8, (T, 1, 2))
    off = rng.uniform(0.19, 0.3, (T, 3, 2)) * np.array([[[-1, -1], [1, -1], [0, 1]]])
    xy = c + off
    z = rng.uniform(-0.9, 0.9, (T, 3, 1))
    pts = np.concatenate([xy, z], axis=2).astype(np.float32).reshape(-1, 3)
    idx = np.arange(3 * T, dtype=np.int32).reshape(-1, 3)
    # window-space bounding boxes: every triangle spans > 128 pixels
    wx = (xy[..., 0] + 1.0) * 0.5 * W
    wy = (xy[..., 1] + 1.0) * 0.5 * H
    big = ((np.floor(wx.max(1)) - np.ceil(wx.min(1))) >= 20) & ((np.floor(wy.max(1)) - np.ceil(wy.min(1))) >= 20)
    assert int(big.sum()) > 16384 + 1000
    s = gi.Scene().object_from_arrays(pts, idx).commit()
    mvp = np.eye(4, dtype=np.float32).reshape(-1)
    _gbuffer_pair(lib, ctx, s, mvp, W, H, stream)  # warm-up: loads the module and kernels
    for _ in range(2):
        free0, free1, (a_pos, a_nrm), (b_pos, b_nrm) = _gbuffer_pair(lib, ctx, s, mvp, W, H, stream)
        assert free0 == free1, f"the call changed free device memory by {free0 - free1} bytes"
        assert np.array_equal(a_pos.view(np.uint32), b_pos.view(np.uint32))
        assert np.array_equal(a_nrm.view(np.uint32), b_nrm.view(np.uint32))
        assert (b_pos.reshape(-1, 4)[:, 3] == 1.0).sum() > 0.9 * W * H  # the triangles cover the image
    ctx.close()


def test_noalloc_gbuffer_rejects_images_above_its_limit():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = api.load()
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    idx = torch.zeros(3, dtype=torch.int32, device="cuda")
    st = _noalloc(lib, dummy, dummy, 1, idx, 1, np.eye(4, dtype=np.float32).reshape(-1), 1025, 1024, dummy,
                  dummy, torch.cuda.current_stream())
    assert st == api.GI_ERR_CAPACITY
    assert b"1048576" in lib.gi_last_error_string()
