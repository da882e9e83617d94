"""Moment soft shadows (SAVSM, VSSM, ESSM, MSSM) in the CPU oracle.

The oracle's restatement of SoftShadowMapping's moment path is pinned
against a second, independent numpy float32 restatement
(tests/soft_moment_ref.py): the light-side maps (moment map, summed-area
table, min-max levels) texel for texel and the per-pixel lookups probe by
probe, bit for bit except ESSM, whose exp goes through different libm
implementations (numpy's and glibc's) and is compared within a tolerance.
The SAT is also checked against a float64 2-D cumulative sum, and the
reference's iteration count logf(w) / logf(2) against log2(w).
"""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api
import soft_moment_ref as ref

TECHS = {"savsm": api.GI_TECH_SAVSM, "vssm": api.GI_TECH_VSSM, "essm": api.GI_TECH_ESSM, "mssm": api.GI_TECH_MSSM}
IDENTITY = np.eye(4, dtype=np.float32).reshape(-1)


def blocker_scene(S, seed, empty_frac=0.02):
    """A receiver plane at window depth 0.985 under a few nearer rectangles, some texels empty (1.0)."""
    rng = np.random.default_rng(seed)
    d = np.full((S, S), 0.985, np.float32)
    for _ in range(4):
        x0, y0 = rng.integers(0, S - S // 4, 2)
        w, h = rng.integers(S // 8, S // 3, 2)
        d[y0:y0 + h, x0:x0 + w] = np.float32(0.95 + 0.02 * rng.random())
    d += (rng.random((S, S)) * 1e-3).astype(np.float32)
    d[rng.random((S, S)) < empty_frac] = 1.0
    return d.astype(np.float32)


def params(tech, sat, **kw):
    p = gi.ShadowParams.defaults(TECHS[tech])
    p.summed_area_table = sat
    p.pretest = api.GI_PRETEST_OFF
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def probe_frame():
    return gi.Frame(IDENTITY, IDENTITY, IDENTITY, IDENTITY, np.eye(3, dtype=np.float32).reshape(-1),
                    np.zeros(3, np.float32))


def oracle_probes(p, depth, probes):
    """Visibility of synthetic G-buffer pixels whose light-space coordinates are the probes (s, t, z)."""
    S = depth.shape[0]
    n = len(probes)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = probes
    pos[:, 3] = 1.0
    nrm = np.tile(np.array([0, 0, 1, 1], np.float32), (n, 1))
    return oracle.visibility(p.to_c(probe_frame()), depth.reshape(-1), S, S, pos, nrm, n, 1)


def random_probes(n, seed, zs=(0.96, 0.975, 0.98, 0.99, 0.995)):
    rng = np.random.default_rng(seed)
    st = rng.random((n, 2)).astype(np.float32) * np.float32(1.1) - np.float32(0.05)
    z = np.array(zs, np.float32)[rng.integers(0, len(zs), n)]
    return np.concatenate([st, z[:, None]], 1).astype(np.float32)


# ---- light-side maps -----------------------------------------------------------
@pytest.mark.parametrize("S", [1, 2, 4, 8, 64, 256, 1024, 2048, 4096, 16384])
def test_sat_iterations_are_log2(S):
    assert ref.sat_iterations(S) == int(np.log2(S))


@pytest.mark.parametrize("tech", list(TECHS))
@pytest.mark.parametrize("S,T", [(64, 64), (48, 40), (128, 128)])
def test_moment_map_matches_numpy(tech, S, T):
    d = blocker_scene(max(S, T), 3)[:T, :S].copy()
    got = oracle.soft_moment_map(params(tech, False).to_c(None), d, S, T)
    want = ref.moment_map(tech, d)
    if tech == "essm":
        np.testing.assert_allclose(got, want, rtol=2e-6, atol=0)
    else:
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    empty = d >= 1.0
    assert (got[empty] == 0).all() and empty.any()


@pytest.mark.parametrize("tech", ["savsm", "mssm"])
@pytest.mark.parametrize("S,T", [(64, 64), (48, 40), (256, 256), (100, 37)])
def test_summed_area_table_matches_numpy(tech, S, T):
    d = blocker_scene(max(S, T), 5)[:T, :S].copy()
    got = oracle.soft_moment_map(params(tech, True).to_c(None), d, S, T)
    want = ref.summed_area_table(ref.moment_map(tech, d))
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("S", [64, 256])
def test_summed_area_table_is_the_prefix_sum(S):
    # with log2(S) iterations every texel holds the sum over [0, x] x [0, y]
    d = blocker_scene(S, 9)
    m = oracle.soft_moment_map(params("savsm", False).to_c(None), d, S, S).astype(np.float64)
    sat = oracle.soft_moment_map(params("savsm", True).to_c(None), d, S, S)
    exact = m.cumsum(0).cumsum(1)
    scale = np.abs(m).cumsum(0).cumsum(1) + 1e-30
    assert (np.abs(sat - exact) / scale).max() < 2e-6


def test_summed_area_table_of_a_non_power_of_two_width_stops_short():
    # 100 columns: int(logf(100) / logf(2)) = 6 iterations cover offsets up
    # to 63, so x >= 64 sums only the last 64 columns, as the reference does
    S = T = 100
    d = blocker_scene(S, 11)
    m = oracle.soft_moment_map(params("savsm", False).to_c(None), d, S, T).astype(np.float64)
    sat = oracle.soft_moment_map(params("savsm", True).to_c(None), d, S, T)
    assert ref.sat_iterations(S) == 6
    window = m.cumsum(0).cumsum(1)
    window[:, 64:] -= window[:, :S - 64]
    window[64:] -= window[:T - 64]
    np.testing.assert_allclose(sat, window, rtol=0, atol=1e-3)


@pytest.mark.parametrize("S,alpha,beta", [(64, 0.0, 0.0), (256, 0.001, -0.002), (32, -0.01, 0.0)])
def test_min_max_levels_match_numpy(S, alpha, beta):
    d = blocker_scene(S, 13)
    d[3, 5] = 0.0  # PrepareMinMax turns a zero depth into min 1
    p = params("vssm", False, hsm_alpha=alpha, hsm_beta=beta).to_c(None)
    levels = ref.hsm_levels(d, alpha, beta, 4)
    for k in range(5):
        got = oracle.hierarchical_shadow_map(p, d, S, S, k)
        np.testing.assert_array_equal(got.view(np.uint32), levels[k].view(np.uint32), err_msg=f"level {k}")
    assert levels[0][3, 5, 0] == np.float32(1.0) + np.float32(alpha)


def test_min_max_level_reads_the_diagonal_neighbours():
    # MinMax.frag's reads sit one output texel (two input texels) off the
    # centre, so a single deep texel reaches the min of the output texels
    # whose diagonal reads cover it, not the one above it
    S = 16
    d = np.full((S, S), 0.9, np.float32)
    d[8, 8] = 0.1
    lv = oracle.hierarchical_shadow_map(params("vssm", False).to_c(None), d, S, S, 1)
    hit = np.argwhere(lv[..., 0] < 0.9)
    assert (4, 4) not in {tuple(h) for h in hit}
    assert {(3, 3), (5, 5), (3, 5), (5, 3)} <= {tuple(h) for h in hit}


# ---- lookups --------------------------------------------------------------------
@pytest.mark.parametrize("sat", [False, True])
@pytest.mark.parametrize("tech", list(TECHS))
@pytest.mark.parametrize("S", [64, 256])
def test_lookups_match_numpy(tech, sat, S):
    d = blocker_scene(S, 17)
    # the SAT branch divides the box sum by SATFilterSize^2 = (K / 2)^2, the
    # texel count of a box a few texels wide (PlausibleSoftShadow.frag:
    # 404-417): a light radius of 0.625 keeps the boxes near that size
    R = 0.625 if sat else 0.5
    p = params(tech, sat, pcss_min_blocker_depth=0.9, light_radius=R)
    probes = random_probes(240, 19, zs=(0.975, 0.985, 0.99))
    got = oracle_probes(p, d, probes)
    pr = ref.Probe(tech, d, sat=sat, light_radius=R, min_blocker=0.9)
    want = np.array([pr(*q) for q in probes], np.float32)
    if tech == "essm":
        close = np.isclose(got, want, rtol=0, atol=1e-4) | (np.isnan(got) & np.isnan(want))
        assert close.mean() >= 0.98, np.argwhere(~close)
    else:
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    fin = got[np.isfinite(got)]
    assert len(np.unique(fin)) >= 2
    if tech in ("savsm", "mssm") and not sat:  # penumbra values, not only lit / umbra
        assert ((fin > 0.25) & (fin < 1.0)).sum() >= 5


@pytest.mark.parametrize("tech", list(TECHS))
def test_blocker_depth_gate_keeps_pixels_lit(tech):
    # computePenumbraWidth returns 0 below an average blocker depth of 0.99
    # (PlausibleSoftShadow.frag:368): with the reference's gate every probe
    # over these 0.95-0.97 blockers is lit, except that VSSM's min-max
    # classification answers first (lit or the intensity)
    d = blocker_scene(64, 23)
    got = oracle_probes(params(tech, False), d, random_probes(64, 29, zs=(0.975, 0.99)))
    if tech == "vssm":
        assert np.isin(got, [1.0, np.float32(0.25)]).all() and (got == np.float32(0.25)).any()
    else:
        assert (got == 1.0).all()


def test_vssm_min_max_classification_short_cuts():
    # a receiver in front of everything is classified lit by the min-max
    # map, one behind the whole neighbourhood as umbra (the intensity)
    S = 64
    d = np.full((S, S), 0.95, np.float32)
    p = params("vssm", False, pcss_min_blocker_depth=0.9)
    got = oracle_probes(p, d, np.array([[0.5, 0.5, 0.9], [0.5, 0.5, 0.999]], np.float32))
    assert got[0] == 1.0 and got[1] == np.float32(0.25)
