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


def _mats(fr):
    return [np.ascontiguousarray(x, np.float32) for x in (fr.light_mvp_biased, fr.camera_mv, fr.normal_matrix,
                                                          fr.light_position)]


@pytest.fixture(scope="module")
def lib_all(lib):
    P, I, F = C.c_void_p, C.c_int, C.c_float
    lib.ref_shadow.argtypes = [I, P, I, P, P, I, I, P, P, P, P, F, I, I, P]
    lib.ref_rbsm.argtypes = [I, I, P, I, P, P, I, I, P, P, P, P, P, F, F, I, I, I, P, P]
    lib.ref_rbssm.argtypes = [P, I, P, P, I, I, P, P, P, P, F, F, I, I, I, I, I, I, P]
    for f in (lib.ref_shadow, lib.ref_rbsm, lib.ref_rbssm):
        f.restype = None
    return lib


@pytest.mark.parametrize("tech,mode,kernel_order,penumbra", [
    (api.GI_TECH_HARD, 0, 7, 1), (api.GI_TECH_PCF, 1, 7, 1), (api.GI_TECH_PCF, 1, 3, 2),
    (api.GI_TECH_PCF_TRICUBIC, 2, 5, 1)], ids=["hard", "pcf 7/1", "pcf 3/2", "tricubic 5/1"])
def test_hard_and_pcf_equal_the_reference_shader(lib_all, frame, tech, mode, kernel_order, penumbra):
    """ShadowMapping's Shadow.frag: the naive hard test and PCF's float loop,
    bilinear and tricubic (textureBicubic), pre-test included."""
    fr, depth, pos, nrm = frame
    p = gi.ShadowParams.defaults(tech)
    p.kernel_order, p.penumbra_size = kernel_order, penumbra
    got = oracle.visibility(p.to_c(fr), depth, S, S, pos, nrm, W, H)
    want = np.empty(W * H, np.float32)
    lib_all.ref_shadow(mode, _ptr(depth), S, _ptr(pos), _ptr(nrm), W, H, *(_ptr(x) for x in _mats(fr)),
                       p.shadow_intensity, kernel_order, penumbra, _ptr(want))
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {W * H} pixels differ"


RBSM = [  # technique, shader (0 non-conservative, 1 conservative, 2 filtered), mode (0 SMSR, 1 RPCF)
    (api.GI_TECH_SMSR_NONCONSERVATIVE, 0, 0), (api.GI_TECH_RPCF_SMSR, 0, 1), (api.GI_TECH_RSMSS, 2, 1),
    (api.GI_TECH_SMSR_CONSERVATIVE, 1, 0), (api.GI_TECH_RPCF_CONSERVATIVE, 1, 1)]


@pytest.mark.parametrize("tech,shader,mode", RBSM,
                         ids=["smsr", "rpcf+smsr", "rsmss", "conservative smsr", "conservative rpcf"])
@pytest.mark.parametrize("threshold", [0.0, 1e-2])
def test_rbsm_equals_the_reference_shaders(lib_all, frame, tech, shader, mode, threshold):
    """NonConservativeSMSR.frag, ConservativeSMSR.frag and FilteredRBSM.frag."""
    fr, depth, pos, nrm = frame
    p = gi.ShadowParams.defaults(tech)
    p.max_search, p.depth_threshold, p.kernel_order, p.penumbra_size = 16, threshold, 3, 1
    got = oracle.visibility(p.to_c(fr), depth, S, S, pos, nrm, W, H)
    out4 = np.empty(W * H * 4, np.float32)
    cmvp = np.ascontiguousarray(fr.camera_mvp, np.float32)
    lf, mv, nm, lp = _mats(fr)
    lib_all.ref_rbsm(shader, mode, _ptr(depth), S, _ptr(pos), _ptr(nrm), W, H, _ptr(lf), _ptr(mv), _ptr(cmvp),
                     _ptr(nm), _ptr(lp), p.shadow_intensity, threshold, 16, 3, 1, _ptr(out4), None)
    want = out4.reshape(-1, 4)[:, 0].copy()
    want[pos.reshape(-1, 4)[:, 0] == 0] = 0.0  # background: the visibility target's clear value
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {W * H} pixels differ"


def test_edtsm_inputs_equal_the_reference_shader(lib_all, frame):
    """The EDTSM outputs of NonConservativeSMSR.frag: (shadow, depth,
    pre-test, 1) and the clip position."""
    fr, depth, pos, nrm = frame
    p = gi.ShadowParams.defaults(api.GI_TECH_SMSR_NONCONSERVATIVE)
    c = p.to_c(fr)
    vis = oracle.visibility(c, depth, S, S, pos, nrm, W, H)
    image, position = oracle.edt_inputs(c, fr.camera_mvp, pos, nrm, vis, W, H)
    out4, pos4 = np.empty(W * H * 4, np.float32), np.empty(W * H * 4, np.float32)
    cmvp = np.ascontiguousarray(fr.camera_mvp, np.float32)
    lf, mv, nm, lp = _mats(fr)
    lib_all.ref_rbsm(0, 2, _ptr(depth), S, _ptr(pos), _ptr(nrm), W, H, _ptr(lf), _ptr(mv), _ptr(cmvp), _ptr(nm),
                     _ptr(lp), p.shadow_intensity, p.depth_threshold, p.max_search, p.kernel_order, p.penumbra_size,
                     _ptr(out4), _ptr(pos4))
    assert np.array_equal(image.reshape(-1).view(np.uint32), out4.view(np.uint32))
    assert np.array_equal(position.reshape(-1).view(np.uint32), pos4.view(np.uint32))


@pytest.mark.parametrize("blocker,kernel,radius,threshold", [(7, 15, 4, 0.0), (5, 9, 12, 0.0), (3, 5, 20, 1e-2)])
def test_rbssm_equals_the_reference_shader(lib_all, frame, blocker, kernel, radius, threshold):
    """SoftShadowMapping's RBSSM.frag (1,378 lines) whole."""
    fr, depth, pos, nrm = frame
    p = gi.ShadowParams.defaults(api.GI_TECH_RBSSM)
    p.blocker_search_size, p.kernel_size, p.light_radius = blocker, kernel, float(radius)
    p.pcss_min_blocker_depth, p.znear, p.depth_threshold = 0.99, 1.0, threshold
    got = oracle.visibility(p.to_c(fr), depth, S, S, pos, nrm, W, H)
    want = np.empty(W * H, np.float32)
    lib_all.ref_rbssm(_ptr(depth), S, _ptr(pos), _ptr(nrm), W, H, *(_ptr(x) for x in _mats(fr)), p.shadow_intensity,
                      threshold, p.max_search, blocker, kernel, radius, 1, 1000, _ptr(want))
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {W * H} pixels differ"
    fg = want[pos.reshape(-1, 4)[:, 0] != 0]
    assert ((fg > p.shadow_intensity) & (fg < 1.0)).sum() >= 10


def test_phong_equals_the_reference_shader(lib_all, frame):
    """ShadowMapping's PhongShading.frag (shadeScene) over the G-buffer, with
    visibility values of every kind and per-pixel colours."""
    fr, depth, pos, nrm = frame
    lib_all.ref_phong.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_int] + [C.c_void_p] * 3 + [C.c_float, C.c_void_p]
    lib_all.ref_phong.restype = None
    p = gi.ShadowParams.defaults(api.GI_TECH_HARD)
    c = p.to_c(fr)
    rng = np.random.default_rng(3)
    vis = rng.choice(np.array([0.0, 0.25, 1.0, 0.55], np.float32), W * H).astype(np.float32)
    color = rng.random(W * H * 4, dtype=np.float32)
    got = oracle.phong_shade(c, pos, nrm, vis, W, H, color)
    want = np.empty(W * H * 4, np.float32)
    _, mv, nm, lp = _mats(fr)
    lib_all.ref_phong(_ptr(pos), _ptr(nrm), _ptr(vis), _ptr(color), W, H, _ptr(mv), _ptr(nm), _ptr(lp),
                      p.shadow_intensity, _ptr(want))
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {W * H * 4} values differ"


@pytest.mark.parametrize("tech,mode", [(api.GI_TECH_VSM, 3), (api.GI_TECH_ESM, 4), (api.GI_TECH_EVSM, 5),
                                       (api.GI_TECH_MSM, 6)], ids=["VSM", "ESM", "EVSM", "MSM"])
def test_moment_lookups_equal_the_reference_shader(lib_all, tech, mode):
    """Shadow.frag's varianceShadowMapping, exponentialShadowMapping,
    exponentialVarianceShadowMapping and hamburger4MSM over the blurred
    moment target (made by tests/moment_ref.py, which equals the oracle's
    own, texel for texel), read bilinearly."""
    import moment_ref
    from globalillumination_gb300 import scenes

    Wm, Sm = 48, 96
    w = scenes.pcss_1080p(width=Wm, height=Wm, map_size=Sm, spheres=10)
    fr = gi.frame_setup(w.light, w.camera)
    p, n, i = w.scene.arrays()
    w.scene.close()
    mp = w.map_params
    depth = oracle.shadow_map(p, i, fr.light_mvp, Sm, Sm, mp.bias_mode, mp.constant_bias, mp.offset_factor,
                              mp.offset_units)
    pos, nrm = oracle.gbuffer(p, n, i, fr.camera_mvp, Wm, Wm)
    prm = gi.ShadowParams.defaults(tech)
    got = oracle.visibility(prm.to_c(fr), depth, Sm, Sm, pos, nrm, Wm, Wm)
    moments = np.ascontiguousarray(moment_ref.filtered(tech, depth, Sm, Wm), np.float32)
    _, mqi = moment_ref.quantization()
    mqi = np.array(mqi, np.float32)
    lib_all.ref_shadow_moments.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p,
                                           C.c_float, C.c_void_p]
    lib_all.ref_shadow_moments.restype = None
    want = np.empty(Wm * Wm, np.float32)
    lib_all.ref_shadow_moments(mode, _ptr(moments), Wm, _ptr(pos), _ptr(nrm), Wm, Wm, *(_ptr(x) for x in _mats(fr)),
                               prm.shadow_intensity, _ptr(mqi), float(moment_ref.TQ0), _ptr(want))
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {Wm * Wm} pixels differ"
    fg = want[pos.reshape(-1, 4)[:, 0] != 0]
    assert ((fg > prm.shadow_intensity) & (fg < 1.0)).any()


@pytest.mark.parametrize("tech,mode", [(api.GI_TECH_SAVSM, 0), (api.GI_TECH_ESSM, 1)], ids=["SAVSM", "ESSM"])
@pytest.mark.parametrize("sat", [False, True], ids=["moment map", "SAT"])
def test_soft_moments_equal_the_reference_shader(lib_all, frame, tech, mode, sat):
    """PlausibleSoftShadow.frag's summedAreaVarianceShadowMapping and
    exponentialSoftShadowMapping over the oracle's moment map or its SAT
    (which tests/soft_moment_ref.py pins texel for texel), read bilinearly."""
    fr, depth, pos, nrm = frame
    prm = gi.ShadowParams.defaults(tech)
    prm.blocker_search_size, prm.kernel_size, prm.light_radius = 7, 7, 4.0
    prm.pcss_min_blocker_depth, prm.znear, prm.summed_area_table = 0.99, 1.0, sat
    c = prm.to_c(fr)
    got = oracle.visibility(c, depth, S, S, pos, nrm, W, H)
    moments = np.ascontiguousarray(oracle.soft_moment_map(c, depth, S, S), np.float32)
    lib_all.ref_soft_moments.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                         C.c_int, C.c_int, C.c_int, C.c_void_p]
    lib_all.ref_soft_moments.restype = None
    want = np.empty(W * H, np.float32)
    lib_all.ref_soft_moments(mode, int(sat), _ptr(depth), _ptr(moments), S, _ptr(pos), _ptr(nrm), W, H,
                             *(_ptr(x) for x in _mats(fr)), prm.shadow_intensity, 7, 7, 4, _ptr(want))
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {W * H} pixels differ"
