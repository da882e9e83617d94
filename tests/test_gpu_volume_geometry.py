"""gi_shadow_volume_geometry on the GPU against the reference's ShadowVolume::build.

The fixture (tests/golden/scene_pin.npz, made by
tests/golden/make_scene_golden.py from the reference's own
ShadowVolumes/src/ShadowVolume.cpp:15-114 compiled here) holds Door's mesh
and the triangles the reference builds from it for two lights; the kernel
emits the same triangles through the device function the stencil pass
rasterises, so they must match bit for bit.  A larger synthetic scene is
checked against the oracle.
"""
import os

import numpy as np
import pytest

import globalillumination_gb300 as gi
import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scene_pin.npz")


def _device_volume(ctx, s, p, n, ix, L):
    import torch

    p, n, ix = (np.ascontiguousarray(a) for a in (p, n, ix))
    s.upload_from(ctx, p.ctypes.data, n.ctypes.data, p.shape[0], ix.ctypes.data, ix.shape[0])
    out = torch.full((6 * ix.shape[0] * 9,), float("nan"), dtype=torch.float32, device="cuda")
    gi.shadow_volume_geometry(ctx, s, L, out, 100.0)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(-1, 3, 3)


@pytest.mark.parametrize("tag", ["le", "side"])
def test_volume_geometry_equals_reference_shadow_volume_build(cuda_ctx, tag):
    gold = np.load(GOLD)
    p, n, ix = gold["door_points"], gold["door_normals"], gold["door_indices"]
    s = gi.Scene().object_from_arrays(p, ix).commit()
    got = _device_volume(cuda_ctx, s, p, n, ix, gold[f"door_volume_{tag}_light"])
    want = gold[f"door_volume_{tag}"]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_volume_geometry_equals_oracle_on_sphere_field(cuda_ctx):
    s = gi.Scene().ground(10.0).icosphere_field(40, 3, (-8, 0.2, -8), (8, 3, 8), 0.2, 1.0, 0x5EED0043)
    p, n, ix = s.arrays()
    for L in ((0.0, 12.0, 0.0), (-7.5, 4.25, 3.0)):
        got = _device_volume(cuda_ctx, s, p, n, ix, L)
        want = oracle.shadow_volume_geometry(p, n, ix, np.array(L, np.float32), 100.0)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
