"""The C++ oracle's hard test, PCF and PCSS (grid and Poisson) against a
second restatement of the same shader text in numpy float32
(tests/shadow_lookup_ref.py), bit for bit, on G-buffer pixels and a light
map that the oracle rasterises from a sphere-field scene."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api
from globalillumination_gb300 import scenes

import shadow_lookup_ref as ref

W, H, S = 96, 54, 128


@pytest.fixture(scope="module")
def world():
    w = scenes.pcss_1080p(width=W, height=H, map_size=S, spheres=24)
    fr = gi.frame_setup(w.light, w.camera)
    p, n, i = w.scene.arrays()
    mp = w.map_params
    depth = oracle.shadow_map(p, i, fr.light_mvp, S, S, mp.bias_mode, mp.constant_bias, mp.offset_factor,
                              mp.offset_units)
    pos, nrm = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    pos, nrm = pos.reshape(-1, 4), nrm.reshape(-1, 4)
    rng = np.random.default_rng(0x5EED)
    fg = np.flatnonzero(pos[:, 0] != 0)
    bg = np.flatnonzero(pos[:, 0] == 0)
    pick = np.concatenate([rng.choice(fg, 400, replace=False), rng.choice(bg, 4, replace=False)])
    w.scene.close()
    return fr, depth, pos[pick].copy(), nrm[pick].copy(), pos, nrm


@pytest.fixture(scope="module")
def world_probes(world):
    return world[:4]


CASES = [
    ("hard", api.GI_TECH_HARD, {}),
    ("hard, no pre-test", api.GI_TECH_HARD, {"pretest": api.GI_PRETEST_OFF}),
    ("hard, soft app", api.GI_TECH_HARD_SOFTAPP, {}),
    ("pcf 7 / 1", api.GI_TECH_PCF, {"kernel_order": 7, "penumbra_size": 1}),
    ("pcf 3 / 2", api.GI_TECH_PCF, {"kernel_order": 3, "penumbra_size": 2}),
    ("pcf tricubic 5 / 1", api.GI_TECH_PCF_TRICUBIC, {"kernel_order": 5, "penumbra_size": 1}),
    ("pcss grid 7 / 15", api.GI_TECH_PCSS_GRID,
     {"blocker_search_size": 7, "kernel_size": 15, "light_radius": 4.0, "pcss_min_blocker_depth": 0.0}),
    ("pcss grid 4 / 6, cut-off", api.GI_TECH_PCSS_GRID,
     {"blocker_search_size": 4, "kernel_size": 6, "light_radius": 2.5, "pcss_min_blocker_depth": 0.99}),
    ("pcss poisson 16 / 32", api.GI_TECH_PCSS_POISSON,
     {"poisson_blocker_taps": 16, "poisson_filter_taps": 32, "kernel_size": 15, "light_radius": 4.0,
      "pcss_min_blocker_depth": 0.0}),
    ("pcss poisson 8 / 12, no pre-test", api.GI_TECH_PCSS_POISSON,
     {"poisson_blocker_taps": 8, "poisson_filter_taps": 12, "kernel_size": 9, "light_radius": 6.0,
      "pcss_min_blocker_depth": 0.0, "pretest": api.GI_PRETEST_OFF}),
]


@pytest.mark.parametrize("name,tech,fields", CASES, ids=[c[0] for c in CASES])
def test_oracle_lookups_equal_the_second_restatement(world_probes, name, tech, fields):
    fr, depth, pos, nrm = world_probes
    p = gi.ShadowParams.defaults(tech)
    for k, v in fields.items():
        setattr(p, k, v)
    c = p.to_c(fr)
    bt = gi.poisson_table(p.poisson_blocker_taps)
    ft = gi.poisson_table(p.poisson_filter_taps)
    tab = np.concatenate([bt.reshape(-1), ft.reshape(-1)])
    got = oracle.visibility(c, depth, S, S, pos.reshape(-1), nrm.reshape(-1), len(pos), 1, tab)
    rp = ref.params_of(c)
    taps_b = [(np.float32(x), np.float32(y)) for x, y in bt]
    taps_f = [(np.float32(x), np.float32(y)) for x, y in ft]
    want = np.array([ref.shade(rp, depth, S, S, [np.float32(v) for v in pos[k]], [np.float32(v) for v in nrm[k]],
                               taps_b, taps_f) for k in range(len(pos))], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        f"{name}: {int((got != want).sum())} of {len(pos)} pixels differ"
    fgv = want[pos[:, 0] != 0]
    if "cut-off" in name:
        # every blocker of this scene lies below the reference's 0.99 cut-off,
        # so PCSS returns fully lit wherever the pre-test passes
        assert set(np.unique(fgv).tolist()) <= {1.0, float(np.float32(p.shadow_intensity))}
        return
    # the probes cover lit, shadowed and (for the soft techniques) partly lit pixels
    assert (fgv == 1.0).any() and (fgv < 1.0).any()
    if tech in (api.GI_TECH_PCF, api.GI_TECH_PCF_TRICUBIC, api.GI_TECH_PCSS_GRID, api.GI_TECH_PCSS_POISSON):
        assert ((fgv > p.shadow_intensity) & (fgv < 1.0)).any(), "no partly lit pixel among the probes"


def test_receiver_on_the_stored_depth_is_lit(world_probes):
    """Shadow.frag's test is z <= depth: a receiver whose texel holds exactly
    its own depth is lit, in the oracle and in the restatement."""
    fr, depth, pos, nrm = world_probes
    p = gi.ShadowParams.defaults(api.GI_TECH_HARD)
    p.pretest = api.GI_PRETEST_OFF
    c = p.to_c(fr)
    rp = ref.params_of(c)
    on_surface = depth.copy()
    fg = [k for k in range(len(pos)) if pos[k, 0] != 0]
    for k in fg:
        v = [np.float32(x) for x in pos[k]]
        sc = ref.mat4_mul(rp["light_mvp_biased"], v)
        s, t, z = sc[0] / sc[3], sc[1] / sc[3], sc[2] / sc[3]
        i, j = int(np.floor(s * np.float32(S))), int(np.floor(t * np.float32(S)))
        if 0 <= i < S and 0 <= j < S:
            on_surface[j * S + i] = z
    got = oracle.visibility(c, on_surface, S, S, pos.reshape(-1), nrm.reshape(-1), len(pos), 1)
    want = np.array([ref.shade(rp, on_surface, S, S, [np.float32(x) for x in pos[k]],
                               [np.float32(x) for x in nrm[k]]) for k in range(len(pos))], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # two probes may share a texel; the one written last is lit for sure
    assert (got[fg] == 1.0).mean() > 0.9


def test_oracle_phong_equals_the_second_restatement(world_probes):
    """Deferred Phong (shadeScene) of the probes, with visibility values of
    every kind (0, the intensity, 1 and fractions) and per-pixel colours."""
    fr, depth, pos, nrm = world_probes
    p = gi.ShadowParams.defaults(api.GI_TECH_HARD)
    c = p.to_c(fr)
    rng = np.random.default_rng(7)
    vis = rng.choice(np.array([0.0, 0.25, 1.0, 0.6, 0.93], np.float32), len(pos)).astype(np.float32)
    color = rng.random((len(pos), 4), dtype=np.float32)
    got = oracle.phong_shade(c, pos.reshape(-1), nrm.reshape(-1), vis, len(pos), 1, color.reshape(-1))
    rp = ref.params_of(c)
    want = np.array([ref.phong(rp, [np.float32(v) for v in pos[k]], [np.float32(v) for v in nrm[k]], vis[k], color[k])
                     for k in range(len(pos))], np.float32).reshape(-1)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_oracle_area_light_truth_equals_the_second_restatement():
    """The uniform area-light ground truth of a 3 x 3 sample grid, every map
    and the G-buffer drawn by the brute-force rasteriser."""
    Wc, Hc, Sm = 48, 28, 64
    w = scenes.pcss_1080p(width=Wc, height=Hc, map_size=Sm, spheres=6)
    views = gi.area_light_samples(w.light, 1.5, 3)
    frames = [gi.frame_setup(v, w.camera) for v in views]
    p, n, i = w.scene.arrays()
    w.scene.close()
    mp = w.map_params
    mvps = np.stack([f.light_mvp for f in frames])
    biased = np.stack([f.light_mvp_biased for f in frames])
    args = (p, n, i, mvps, biased, Sm, mp.bias_mode, mp.constant_bias, mp.offset_factor, mp.offset_units,
            frames[0].camera_mvp, 0.25, Wc, Hc)
    got = oracle.area_light_visibility(*args)
    want = ref.area_light_visibility(*args)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"{int((got != want).sum())} pixels differ"
    assert ((want > 0.25) & (want < 1.0)).any()  # penumbrae present


SMSR_CASES = [
    ("smsr", api.GI_TECH_SMSR_NONCONSERVATIVE, {"max_search": 16, "depth_threshold": 0.0}),
    ("smsr, depth threshold", api.GI_TECH_SMSR_NONCONSERVATIVE, {"max_search": 8, "depth_threshold": 1e-2}),
    ("rpcf + smsr 3 / 1", api.GI_TECH_RPCF_SMSR, {"max_search": 16, "kernel_order": 3, "penumbra_size": 1}),
    ("rpcf + smsr 2 / 2, threshold", api.GI_TECH_RPCF_SMSR,
     {"max_search": 12, "kernel_order": 2, "penumbra_size": 2, "depth_threshold": 1e-2}),
    ("rsmss 3 / 1", api.GI_TECH_RSMSS, {"max_search": 16, "kernel_order": 3, "penumbra_size": 1,
                                         "depth_threshold": 0.0}),
    ("rsmss 5 / 2, threshold", api.GI_TECH_RSMSS,
     {"max_search": 12, "kernel_order": 5, "penumbra_size": 2, "depth_threshold": 1e-2}),
    ("conservative smsr", api.GI_TECH_SMSR_CONSERVATIVE, {"max_search": 16, "depth_threshold": 0.0}),
    ("conservative smsr, threshold", api.GI_TECH_SMSR_CONSERVATIVE, {"max_search": 6, "depth_threshold": 1e-2}),
    ("conservative rpcf 3 / 1", api.GI_TECH_RPCF_CONSERVATIVE,
     {"max_search": 16, "kernel_order": 3, "penumbra_size": 1, "depth_threshold": 0.0}),
    ("conservative rpcf 4 / 2, threshold", api.GI_TECH_RPCF_CONSERVATIVE,
     {"max_search": 10, "kernel_order": 4, "penumbra_size": 2, "depth_threshold": 1e-2}),
]


@pytest.mark.parametrize("name,tech,fields", SMSR_CASES, ids=[c[0] for c in SMSR_CASES])
def test_oracle_smsr_equals_the_second_restatement(world, name, tech, fields):
    """NonConservativeSMSR.frag (SMSR and RPCF + SMSR), FilteredRBSM.frag
    (RSMSS) and ConservativeSMSR.frag (SMSR and RPCF) on the probes, bit for bit, with enough probes on shadow
    edges to exercise the revectorisation."""
    import smsr_ref

    fr, depth, _, _, pos, nrm = world  # every pixel of the frame
    p = gi.ShadowParams.defaults(tech)
    for k, v in fields.items():
        setattr(p, k, v)
    c = p.to_c(fr)
    got = oracle.visibility(c, depth, S, S, pos.reshape(-1), nrm.reshape(-1), len(pos), 1)
    rp = ref.params_of(c)
    conservative = tech in (api.GI_TECH_SMSR_CONSERVATIVE, api.GI_TECH_RPCF_CONSERVATIVE)
    args = (depth, S, S, p.shadow_intensity, p.depth_threshold, p.max_search, p.kernel_order, p.penumbra_size)
    if conservative:
        sm = smsr_ref.ConservativeSmsr(*args)
    else:
        sm = smsr_ref.Smsr(*args, filtered=tech == api.GI_TECH_RSMSS)
    want = []
    for k in range(len(pos)):
        v, nv = [np.float32(x) for x in pos[k]], [np.float32(x) for x in nrm[k]]
        if v[0] == 0:
            want.append(np.float32(0.0))
            continue
        sc = ref.mat4_mul(rp["light_mvp_biased"], v)
        n = [sc[0] / sc[3], sc[1] / sc[3], sc[2] / sc[3], sc[3] / sc[3]]
        shadow = ref.pretest(rp, v, nv)
        if shadow == 1:
            smsr = tech in (api.GI_TECH_SMSR_NONCONSERVATIVE, api.GI_TECH_SMSR_CONSERVATIVE)
            shadow = sm.smsr(n) if smsr else sm.rpcf(n)
        want.append(shadow)
    want = np.array(want, np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        f"{name}: {int((got != want).sum())} of {len(pos)} pixels differ"
    assert sm.discontinuities >= 10, "too few probes on a shadow edge"


@pytest.mark.parametrize("lower_accuracy", [False, True], ids=["full", "lower accuracy"])
def test_oracle_adaptive_area_light_equals_the_second_restatement(lower_accuracy):
    """The adaptive (quad-tree) area-light ground truth: the same samples in
    the same order, the same levels and the same image, every map and the
    G-buffer drawn by the brute-force rasteriser.  The full-accuracy case
    refines to level 3 in several quadrants; the lower-accuracy evaluation
    looks at a quarter-size viewport, so it gets a larger window."""
    import dataclasses

    Wc, Hc, Sm, size, depth = (96, 56, 64, 6.0, 2) if lower_accuracy else (64, 40, 64, 8.0, 3)
    w = scenes.pcss_1080p(width=Wc, height=Hc, map_size=Sm, spheres=1)
    w.scene.close()
    s = gi.Scene()
    s.ground(10.0, 0.0)
    s.icosphere_field(8, 2, (-8.0, 0.2, -8.0), (8.0, 3.0, 8.0), 0.2, 1.0, 0x5EED0001)
    p, n, i = s.arrays()
    s.close()
    mp = w.map_params
    cam = gi.frame_setup(w.light, w.camera).camera_mvp

    def view_mvp(eye, at):
        v = dataclasses.replace(w.light, eye=tuple(eye), at=tuple(at))
        f = gi.frame_setup(v, v)
        return f.light_mvp, f.light_mvp_biased

    args = (p, n, i, w.light.eye, w.light.at, size, depth, view_mvp, Sm, mp.bias_mode, mp.constant_bias,
            mp.offset_factor, mp.offset_units, cam, 0.25, Wc, Hc)
    vis, eyes, levels = oracle.area_light_adaptive(*args, lower_accuracy=lower_accuracy)
    r_vis, r_eyes, r_levels = ref.area_light_adaptive(*args, lower_accuracy=lower_accuracy)
    assert np.array_equal(eyes.view(np.uint32), r_eyes.view(np.uint32))
    assert np.array_equal(levels, r_levels)
    assert np.array_equal(vis.view(np.uint32), r_vis.view(np.uint32)), f"{int((vis != r_vis).sum())} pixels differ"
    assert len(levels) > 4, "the light was refined at least once"
    if not lower_accuracy:
        assert levels.max() == 3.0 and len(levels) > 40


def test_oracle_edt_mean_filter_equals_the_second_restatement():
    """EDTSM's screen-space mean filter on a rendered G-buffer, with shadow
    values of every kind and the pixels' own window depths in channel 1."""
    Wc, Hc = 64, 40
    w = scenes.pcss_1080p(width=Wc, height=Hc, map_size=64, spheres=6)
    fr = gi.frame_setup(w.light, w.camera)
    p, n, i = w.scene.arrays()
    w.scene.close()
    pos, _ = oracle.gbuffer(p, n, i, fr.camera_mvp, Wc, Hc)
    pos = pos.reshape(Hc, Wc, 4)
    rng = np.random.default_rng(11)
    img = np.zeros((Hc, Wc, 4), np.float32)
    img[..., 0] = rng.choice(np.array([0.25, 1.0, 1.0, 0.6], np.float32), (Hc, Wc))
    m = fr.camera_mvp.reshape(4, 4).T  # column-major -> rows
    clip = pos.reshape(-1, 4) @ m.T.astype(np.float64)
    img[..., 1] = (clip[:, 2] / clip[:, 3] * 0.5 + 0.5).reshape(Hc, Wc).astype(np.float32)
    img[pos[..., 0] == 0] = (0.0, 0.0, 0.0, 1.0)
    prm = gi.ShadowParams.defaults(api.GI_TECH_SMSR_NONCONSERVATIVE)
    c = prm.to_c(fr)
    got = oracle.edt_mean_filter(c, img, pos, Wc, Hc)
    want = ref.edt_mean_filter(ref.params_of(c), img, pos, Wc, Hc)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"{int((got != want).sum())} values differ"
    fg = pos[..., 0] != 0
    assert ((got[..., 0] > 0.25) & (got[..., 0] < 1.0) & fg).any()


def test_oracle_edt_inputs_equal_the_second_restatement(world):
    """The image and position targets the SMSR shaders write for EDTSM."""
    fr, depth, _, _, pos, nrm = world
    prm = gi.ShadowParams.defaults(api.GI_TECH_SMSR_NONCONSERVATIVE)
    c = prm.to_c(fr)
    rng = np.random.default_rng(5)
    vis = rng.choice(np.array([0.25, 1.0, 0.0], np.float32), len(pos)).astype(np.float32)
    image, position = oracle.edt_inputs(c, fr.camera_mvp, pos.reshape(-1), nrm.reshape(-1), vis, W, H)
    rp = ref.params_of(c)
    for k in range(len(pos)):
        im, po = ref.edt_inputs(rp, fr.camera_mvp, [np.float32(x) for x in pos[k]], [np.float32(x) for x in nrm[k]],
                                vis[k])
        y, x = divmod(k, W)
        assert np.array_equal(image[y, x].view(np.uint32), np.array(im, np.float32).view(np.uint32)), k
        assert np.array_equal(position[y, x].view(np.uint32), np.array(po, np.float32).view(np.uint32)), k
