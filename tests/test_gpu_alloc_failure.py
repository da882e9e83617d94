"""Device allocation failures through the C ABI: GI_ERR_OOM, then recovery.

A fresh context grows its scratch on first use.  Each of its first device
allocations is failed in turn (gi_debug_fail_allocation): the scene upload
or the frame returns GI_ERR_OOM, and once the injection is off the same
context and scene render the frame bit for bit like an untouched context."""
import numpy as np
import pytest

import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes

pytestmark = pytest.mark.gpu


def test_injected_device_failures_return_oom_and_context_recovers():
    import torch

    w = scenes.hard_pcf_1024(width=320, height=240, map_size=256)
    fr = gi.frame_setup(w.light, w.camera)
    S, W, H = w.map_params.width, w.camera.width, w.camera.height
    good = gi.Context(0)
    w.scene.upload(good)
    ref = gi.allocate_frame(S, S, W, H)
    gi.render_frame(good, w.scene, fr, w.map_params, w.params, W, H, ref)
    torch.cuda.synchronize()
    seen_oom = 0
    try:
        for k in range(64):
            ctx = gi.Context(0)
            scene = scenes.hard_pcf_1024(width=320, height=240, map_size=256).scene
            out = gi.allocate_frame(S, S, W, H)
            gi.debug_fail_allocation(k)
            failed = False
            try:
                scene.upload(ctx)
                gi.render_frame(ctx, scene, fr, w.map_params, w.params, W, H, out)
            except gi.GIError as e:
                assert e.status == api.GI_ERR_OOM, e
                failed = True
                seen_oom += 1
            gi.debug_fail_allocation(-1)
            # recovery on the same context and scene
            scene.upload(ctx)
            gi.render_frame(ctx, scene, fr, w.map_params, w.params, W, H, out)
            torch.cuda.synchronize()
            assert torch.equal(out.vis.view(torch.int32), ref.vis.view(torch.int32)), k
            assert torch.equal(out.depth.view(torch.int32), ref.depth.view(torch.int32)), k
            ctx.close()
            if not failed:
                break
    finally:
        gi.debug_fail_allocation(-1)
    assert seen_oom >= 3
    good.close()
