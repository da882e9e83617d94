"""gi_context_set_frame_graph: repeated gi_render_frame calls replay one
captured CUDA graph, with the same bits as the direct launches.

The frame path's launch sequence depends only on its arguments, the scene's
device copy, the context's settings and the library's buffer epoch; each
test compares graph-mode frames with frames of a second context that
launches directly.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import globalillumination_gb300 as gi  # noqa: E402
from globalillumination_gb300 import scenes  # noqa: E402

pytestmark = pytest.mark.gpu


def _world(W=320, H=184, S=512):
    return scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=24)


def _render(ctx, w, fr, bufs, stream):
    gi.render_frame(ctx, w.scene, fr, w.map_params, w.params, w.camera.width, w.camera.height, bufs, stream)
    torch.cuda.synchronize()
    return bufs.vis.clone(), bufs.depth.clone()


@pytest.fixture
def pair():
    g = gi.Context(0)
    d = gi.Context(0)
    g.set_frame_graph(True)
    yield g, d
    g.close()
    d.close()


def test_repeats_replay_with_direct_bits(pair):
    g, d = pair
    w = _world()
    fr = gi.frame_setup(w.light, w.camera)
    stream = torch.cuda.current_stream()
    w.scene.upload(g, stream)
    S = w.map_params.width
    bg = gi.allocate_frame(S, S, w.camera.width, w.camera.height)
    bd = gi.allocate_frame(S, S, w.camera.width, w.camera.height)
    ref_vis, ref_depth = _render(d, w, fr, bd, stream)
    per_frame = None
    for k in range(4):  # direct, capture + launch, replay, replay
        bg.vis.zero_()
        l0 = g.launch_count
        vis, depth = _render(g, w, fr, bg, stream)
        n = g.launch_count - l0
        per_frame = per_frame or n
        assert n == per_frame, "every call counts the kernels it runs"
        assert torch.equal(vis, ref_vis), f"call {k}: visibility differs from the direct launch"
        assert torch.equal(depth, ref_depth), f"call {k}: light map differs from the direct launch"


def test_new_arguments_and_new_scene_contents(pair):
    g, d = pair
    stream = torch.cuda.current_stream()
    w = _world()
    S = w.map_params.width
    bg = gi.allocate_frame(S, S, w.camera.width, w.camera.height)
    bd = gi.allocate_frame(S, S, w.camera.width, w.camera.height)
    w.scene.upload(g, stream)
    fr = gi.frame_setup(w.light, w.camera)
    for _ in range(3):
        _render(g, w, fr, bg, stream)
    # another light position: a new signature, then its own graph
    w.light.eye = (w.light.eye[0] + 0.7, w.light.eye[1], w.light.eye[2] - 0.4)
    fr2 = gi.frame_setup(w.light, w.camera)
    ref = _render(d, w, fr2, bd, stream)
    for _ in range(3):
        assert torch.equal(_render(g, w, fr2, bg, stream)[0], ref[0])
    # other vertex positions of the same size uploaded into the same buffers:
    # the replayed graph reads the new contents
    pts, nrm, idx = w.scene.arrays()
    moved = (pts * np.float32(1.03) + np.float32(0.05)).astype(np.float32)
    hp = torch.from_numpy(moved.reshape(-1).copy()).pin_memory()
    hn = torch.from_numpy(nrm.reshape(-1).copy()).pin_memory()
    hi = torch.from_numpy(idx.reshape(-1).copy()).pin_memory()
    w.scene.upload_from(g, hp.data_ptr(), hn.data_ptr(), pts.shape[0], hi.data_ptr(), idx.shape[0], stream)
    wd = _world()
    wd.scene.upload_from(d, hp.data_ptr(), hn.data_ptr(), pts.shape[0], hi.data_ptr(), idx.shape[0], stream)
    torch.cuda.synchronize()
    ref2 = _render(d, wd, fr2, bd, stream)
    assert not torch.equal(ref2[0], ref[0]), "the moved geometry should change the image"
    for _ in range(2):
        assert torch.equal(_render(g, w, fr2, bg, stream)[0], ref2[0])


def test_reallocation_invalidates_the_graph(pair):
    g, d = pair
    stream = torch.cuda.current_stream()
    small, large = _world(), _world(W=640, H=368, S=1024)
    for w in (small, large):
        w.scene.upload(g, stream)
    frs = {id(w): gi.frame_setup(w.light, w.camera) for w in (small, large)}
    bufs = {id(w): gi.allocate_frame(w.map_params.width, w.map_params.width, w.camera.width, w.camera.height)
            for w in (small, large)}
    refs = {}
    for w in (small, large):
        bd = gi.allocate_frame(w.map_params.width, w.map_params.width, w.camera.width, w.camera.height)
        refs[id(w)] = _render(d, w, frs[id(w)], bd, stream)[0]
    # small frames (graph captured), a larger frame (grows the context's
    # buffers), then small frames again: the old graph must not replay
    for w in (small, small, small, large, small, small, small):
        assert torch.equal(_render(g, w, frs[id(w)], bufs[id(w)], stream)[0], refs[id(w)])


def test_profiling_bypasses_the_graph(pair):
    g, _ = pair
    stream = torch.cuda.current_stream()
    w = _world()
    w.scene.upload(g, stream)
    fr = gi.frame_setup(w.light, w.camera)
    S = w.map_params.width
    b = gi.allocate_frame(S, S, w.camera.width, w.camera.height)
    for _ in range(3):
        ref = _render(g, w, fr, b, stream)[0]
    g.set_profiling(True)
    vis = _render(g, w, fr, b, stream)[0]
    ms = g.phase_ms()
    g.set_profiling(False)
    assert torch.equal(vis, ref)
    assert all(np.isfinite(ms)) and ms[2] > 0


def test_caller_capture_gets_the_launches(pair):
    """With the frame graph on, a call made while the caller captures its own
    stream enqueues the launches themselves (no graph inside the capture);
    replaying the caller's graph gives the direct frame's bits."""
    g, d = pair
    w = _world()
    fr = gi.frame_setup(w.light, w.camera)
    stream = torch.cuda.current_stream()
    w.scene.upload(g, stream)
    S, W, H = w.map_params.width, w.camera.width, w.camera.height
    bg = gi.allocate_frame(S, S, W, H)
    bd = gi.allocate_frame(S, S, W, H)
    ref_vis, ref_depth = _render(d, w, fr, bd, stream)
    for _ in range(3):  # allocations done, the context's own graph built
        _render(g, w, fr, bg, stream)
    bg.vis.zero_()
    bg.depth.zero_()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.graph(graph, stream=side):
        gi.render_frame(g, w.scene, fr, w.map_params, w.params, W, H, bg, torch.cuda.current_stream())
    torch.cuda.synchronize()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(bg.vis, ref_vis)
    assert torch.equal(bg.depth, ref_depth)
    # the context's own frame graph still replays afterwards
    assert torch.equal(_render(g, w, fr, bg, stream)[0], ref_vis)
