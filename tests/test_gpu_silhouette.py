"""Shadow volumes with silhouette extraction against the exact per-triangle volumes.

gi_shadow_volume_counts_silhouette leaves out every pair of coplanar quads
that cancel (ShadowVolume::build extrudes every triangle,
ShadowVolumes/src/ShadowVolume.cpp:15-114; the stencil passes are
ShadowVolumes/src/main.cpp:120-206).  Its counts must equal the exact
path's (itself bit-exact against the oracle) everywhere except at the few
pixels where a left-out pair's two triangulations round differently; the
test bounds those pixels, checks that the lit / shadowed decision (count
== 0) differs on at most as many, and that far fewer volume triangles were
drawn."""
import numpy as np
import pytest

import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api

pytestmark = pytest.mark.gpu


def _scene(kind):
    s = gi.Scene()
    s.ground(10.0, 0.0)
    if kind == "displaced":
        s.displaced_sphere(96, 48, 2.0, 0.3, (0.0, 2.6, 0.0), 0x5EED0004)
        cam = gi.ViewSpec(eye=(0.0, 9.0, -14.0), at=(0.0, 1.5, 0.0), width=640, height=360)
    else:
        s.icosphere_field(24, 2, (-6.0, 0.2, -6.0), (6.0, 2.5, 6.0), 0.3, 1.0, 0x5EED00B7)
        cam = gi.ViewSpec(eye=(0.0, 10.0, -14.0), at=(0.0, 0.5, 0.0), width=640, height=360)
    return s, cam


@pytest.mark.parametrize("kind", ["displaced", "field"])
@pytest.mark.parametrize("light_eye", [(4.9, 7.0, 0.0), (-2.0, 9.0, -5.0)])
@pytest.mark.parametrize("depth_func", [api.GI_DEPTH_LESS, api.GI_DEPTH_LEQUAL])
def test_silhouette_counts_match_exact_counts(cuda_ctx, kind, light_eye, depth_func):
    import torch

    s, cam = _scene(kind)
    W, H = cam.width, cam.height
    light = gi.ViewSpec(eye=light_eye, at=(0.0, 0.0, 0.0), width=64, height=64)
    fr = gi.frame_setup(light, cam)
    s.upload(cuda_ctx)
    exact = torch.empty(W * H, dtype=torch.uint8, device="cuda")
    sil = torch.empty_like(exact)
    d0 = torch.empty(W * H, device="cuda")
    d1 = torch.empty_like(d0)
    gi.shadow_volume_counts(cuda_ctx, s, light.eye, fr.camera_mvp, W, H, exact, d0, depth_func=depth_func)
    drawn = gi.shadow_volume_counts_silhouette(cuda_ctx, s, light.eye, fr.camera_mvp, W, H, sil, d1,
                                               depth_func=depth_func)
    torch.cuda.synchronize()
    T = s.info().num_triangles
    assert 0 < drawn < 6 * T // 4, (drawn, 6 * T)
    assert torch.equal(d0.view(torch.int32), d1.view(torch.int32))  # same prepass
    a, b = exact.cpu().numpy(), sil.cpu().numpy()
    differ = int((a != b).sum())
    lit_differ = int(((a == 0) != (b == 0)).sum())
    assert (a != 0).sum() > 1000
    assert differ <= 0.002 * W * H, (differ, drawn, 6 * T)
    assert lit_differ <= differ
    # a second call reuses the cached adjacency and gives the same counts
    sil2 = torch.empty_like(exact)
    assert gi.shadow_volume_counts_silhouette(cuda_ctx, s, light.eye, fr.camera_mvp, W, H, sil2,
                                              depth_func=depth_func) == drawn
    torch.cuda.synchronize()
    assert torch.equal(sil, sil2)
