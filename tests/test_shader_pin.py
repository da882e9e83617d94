"""The oracle's per-pixel visibility against the reference's OWN fragment
shaders, compiled unmodified as C++ (oracle/ref_shader_pin.cpp over
oracle/glsl_shim.h, built into oracle/_ref/ where the reference tree is
present): the same G-buffer and light map through both, bit for bit.

The light sits far from the scene so that its depths pass the reference
PCSS's 0.99 average-blocker cut-off, and the light radius is a whole number,
as the reference's int uniform is."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api
from oracle.build_oracle import SHADER_PIN_LIB, build_shader_ref

W, H, S = 160, 90, 128


@pytest.fixture(scope="module")
def lib():
    if build_shader_ref() is None or not os.path.exists(SHADER_PIN_LIB):
        pytest.skip("the reference's shaders are not present here")
    lib = C.CDLL(SHADER_PIN_LIB)
    P = C.c_void_p
    lib.ref_pcss.argtypes = [P, C.c_int, P, P, C.c_int, C.c_int, P, P, P, P, C.c_float, C.c_int, C.c_int, C.c_int,
                             C.c_int, C.c_int, P]
    lib.ref_pcss.restype = None
    return lib


@pytest.fixture(scope="module")
def frame():
    s = gi.Scene()
    s.ground(10.0, 0.0)
    s.icosphere_field(24, 3, (-8.0, 0.2, -8.0), (8.0, 3.0, 8.0), 0.5, 1.8, 0x5EED0011)
    p, n, i = s.arrays()
    s.close()
    light = gi.ViewSpec(eye=(0.0, 150.0, 0.0), at=(0.0, 0.0, 0.0), width=S, height=S, fovy_deg=9.5)
    camera = gi.ViewSpec(eye=(0.0, 14.0, -20.0), at=(0.0, 0.0, 0.0), width=W, height=H)
    fr = gi.frame_setup(light, camera)
    depth = oracle.shadow_map(p, i, fr.light_mvp, S, S, api.GI_BIAS_POLYGON_OFFSET, 0.0, 4.0, 20.0)
    pos, nrm = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    return fr, depth, pos, nrm


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("blocker,kernel,radius", [(7, 15, 4), (5, 9, 12), (3, 5, 20), (7, 15, 20)])
def test_pcss_equals_the_reference_shader(lib, frame, blocker, kernel, radius):
    """PlausibleSoftShadow.frag with PCSS = 1 (its blocker search, penumbra
    width with the 0.99 cut-off and filter), pre-test included."""
    fr, depth, pos, nrm = frame
    p = gi.ShadowParams.defaults(api.GI_TECH_PCSS_GRID)
    p.blocker_search_size, p.kernel_size, p.light_radius = blocker, kernel, float(radius)
    p.pcss_min_blocker_depth, p.znear = 0.99, 1.0
    c = p.to_c(fr)
    got = oracle.visibility(c, depth, S, S, pos, nrm, W, H)
    want = np.empty(W * H, np.float32)
    m = [np.ascontiguousarray(x, np.float32) for x in (fr.light_mvp_biased, fr.camera_mv, fr.normal_matrix,
                                                       fr.light_position)]
    lib.ref_pcss(_ptr(depth), S, _ptr(pos), _ptr(nrm), W, H, *(_ptr(x) for x in m), p.shadow_intensity, blocker,
                 kernel, radius, 1, 1000, _ptr(want))
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {W * H} pixels differ"
    fg = want[pos.reshape(-1, 4)[:, 0] != 0]
    assert ((fg > p.shadow_intensity) & (fg < 1.0)).sum() >= 10, "few penumbrae: the cut-off or the light placement"
