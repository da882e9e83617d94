"""The C++ oracle's filtered moment shadow maps (VSM, ESM, EVSM, MSM: moment
target, box reduction, separable 7-tap blur, lookups) against a second
restatement in numpy float32 (tests/moment_ref.py), on every pixel of a
square window over a sphere-field scene, for maps 1x, 2x and 4x the window."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api
from globalillumination_gb300 import scenes

import moment_ref
import shadow_lookup_ref as ref

W = 48


@pytest.fixture(scope="module")
def frame():
    w = scenes.pcss_1080p(width=W, height=W, map_size=W, spheres=10)
    fr = gi.frame_setup(w.light, w.camera)
    p, n, i = w.scene.arrays()
    w.scene.close()
    pos, nrm = oracle.gbuffer(p, n, i, fr.camera_mvp, W, W)
    return fr, p, i, w.map_params, pos.reshape(-1, 4), nrm.reshape(-1, 4)


@pytest.mark.parametrize("tech", [api.GI_TECH_VSM, api.GI_TECH_ESM, api.GI_TECH_EVSM, api.GI_TECH_MSM],
                         ids=["VSM", "ESM", "EVSM", "MSM"])
@pytest.mark.parametrize("scale", [1, 2, 4])
def test_oracle_moment_shadows_equal_the_second_restatement(frame, tech, scale):
    fr, p, i, mp, pos, nrm = frame
    S = W * scale
    v = gi.ViewSpec(eye=(0.0, 12.0, 0.0), at=(0.0, 0.0, 0.0), width=S, height=S, fovy_deg=90.0)
    light_mvp = gi.frame_setup(v, v).light_mvp
    depth = oracle.shadow_map(p, i, light_mvp, S, S, mp.bias_mode, mp.constant_bias, mp.offset_factor,
                              mp.offset_units)
    prm = gi.ShadowParams.defaults(tech)
    c = prm.to_c(fr)
    got = oracle.visibility(c, depth, S, S, pos.reshape(-1), nrm.reshape(-1), W, W)
    mm = moment_ref.filtered(tech, depth, S, W)
    rp = ref.params_of(c)
    want = np.zeros(W * W, np.float32)
    for k in np.flatnonzero(pos[:, 0] != 0):
        vtx, nv = [np.float32(x) for x in pos[k]], [np.float32(x) for x in nrm[k]]
        sc = ref.mat4_mul(rp["light_mvp_biased"], vtx)
        n = [sc[0] / sc[3], sc[1] / sc[3], sc[2] / sc[3], sc[3] / sc[3]]
        shadow = ref.pretest(rp, vtx, nv)
        if sc[3] > 0 and shadow == 1:
            shadow = moment_ref.lookup(tech, mm, W, n, rp["intensity"])
        want[k] = shadow
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{int(diff.sum())} of {W * W} pixels differ"
    fg = want[pos[:, 0] != 0]
    assert ((fg > prm.shadow_intensity) & (fg < 1.0)).any(), "no filtered penumbra among the pixels"
