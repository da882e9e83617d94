"""Known-answer tests of the CPU oracle (no GPU).

The reference has no tests or golden images, so the oracle is pinned here
by answers derived by hand from the rules it restates: the GL raster rules
(coverage, window-space depth, polygon offset, top-left ownership of shared
edges), the fragment-shader quirks (PCF's float loop, PCSS cut-offs,
CLAMP_TO_BORDER, background discard) and the shadow-volume counts.
"""
import numpy as np
import pytest

import oracle
from globalillumination_gb300 import _capi as api
import globalillumination_gb300 as gi

IDENTITY = np.eye(4, dtype=np.float32).reshape(-1)


def ndc(xw, yw, W, H):
    return xw / (W / 2.0) - 1.0, yw / (H / 2.0) - 1.0


def test_single_triangle_depth_is_the_window_plane():
    W = H = 64
    win = [(8.25, 10.5, 0.25), (50.0, 12.75, 0.625), (20.5, 55.25, 0.875)]  # (x_w, y_w, z_w)
    pts = []
    for xw, yw, zw in win:
        x, y = ndc(xw, yw, W, H)
        pts.append((x, y, 2.0 * zw - 1.0))
    pts = np.array(pts, np.float32)
    d = oracle.shadow_map(pts, np.array([[0, 1, 2]]), IDENTITY, W, H).reshape(H, W)
    A = np.array([[w[0], w[1], 1.0] for w in win])
    coef = np.linalg.solve(A, np.array([w[2] for w in win]))
    ys, xs = np.mgrid[0:H, 0:W] + 0.5
    # barycentrics of pixel centres
    P = np.stack([xs, ys], -1)
    v = np.array([w[:2] for w in win])

    def e(a, b):
        return (v[b, 0] - v[a, 0]) * (P[..., 1] - v[a, 1]) - (v[b, 1] - v[a, 1]) * (P[..., 0] - v[a, 0])

    E = np.stack([e(1, 2), e(2, 0), e(0, 1)], -1)
    inside = (E > 1e-9).all(-1)
    boundary = (np.abs(E) <= 1e-9).any(-1)
    plane = coef[0] * xs + coef[1] * ys + coef[2]
    assert (d[inside] < 1.0).all()
    assert (d[~inside & ~boundary] == 1.0).all()
    assert np.abs(d[inside] - plane[inside]).max() < 3e-7
    assert inside.sum() > 600


def test_shared_diagonal_owned_by_one_triangle():
    # square [8, 40]^2 split along y = x, which runs through pixel centres;
    # A (below) has the diagonal as a left edge and owns it, B does not.
    W = H = 64
    corner = {k: ndc(*k, W, H) for k in [(8, 8), (40, 8), (40, 40), (8, 40)]}
    za, zb = 0.2, 0.4
    pts = np.array([[*corner[(8, 8)], za], [*corner[(40, 8)], za], [*corner[(40, 40)], za],
                    [*corner[(8, 8)], zb], [*corner[(40, 40)], zb], [*corner[(8, 40)], zb]], np.float32)
    d = oracle.shadow_map(pts, np.array([[0, 1, 2], [3, 4, 5]]), IDENTITY, W, H).reshape(H, W)
    wa, wb = np.float32(0.5 * za + 0.5), np.float32(0.5 * zb + 0.5)
    for y in range(H):
        for x in range(W):
            if 8 <= x < 40 and 8 <= y < 40:
                assert d[y, x] == (wa if x >= y else wb), (x, y)
            else:
                assert d[y, x] == 1.0, (x, y)


def test_polygon_offset_value():
    W = H = 64
    # z_w rises by 0.25 over 64 pixels in x, flat in y: m = 2^-8; max z_w = 0.5
    # (exponent -1) gives r = 2^-24; offset = 4 m + 20 r.
    win = [(0.0, 0.0, 0.25), (64.0, 0.0, 0.5), (0.0, 64.0, 0.25)]
    pts = np.array([[*ndc(x, y, W, H), 2 * z - 1] for x, y, z in win], np.float32)
    d = oracle.shadow_map(pts, np.array([[0, 1, 2]]), IDENTITY, W, H, api.GI_BIAS_POLYGON_OFFSET,
                          0.0, 4.0, 20.0).reshape(H, W)
    offset = 4.0 * 2.0 ** -8 + 20.0 * 2.0 ** -24
    x, y = 10, 20
    expect = 0.25 + 0.25 * (x + 0.5) / 64.0 + offset
    assert abs(d[y, x] - expect) < 2e-7
    dc = oracle.shadow_map(pts, np.array([[0, 1, 2]]), IDENTITY, W, H, api.GI_BIAS_CONSTANT, 1e-3).reshape(H, W)
    assert abs(dc[y, x] - (0.25 + 0.25 * (x + 0.5) / 64.0 + 1e-3)) < 2e-7


def _probe(tech, depth_map, S, s, t, z, **kw):
    """Visibility of one synthetic G-buffer pixel whose light-space coordinate is (s, t, z)."""
    p = gi.ShadowParams.defaults(tech)
    for k, v in kw.items():
        setattr(p, k, v)
    p.pretest = api.GI_PRETEST_OFF
    fr = gi.Frame(IDENTITY, IDENTITY, IDENTITY, IDENTITY, np.eye(3, dtype=np.float32).reshape(-1),
                  np.zeros(3, np.float32))
    pos = np.array([s, t, z, 1.0], np.float32)
    nrm = np.array([0, 0, 1, 1], np.float32)
    tab = np.concatenate([gi.poisson_table(p.poisson_blocker_taps).reshape(-1),
                          gi.poisson_table(p.poisson_filter_taps).reshape(-1)])
    return float(oracle.visibility(p.to_c(fr), depth_map, S, S, pos, nrm, 1, 1, tab)[0])


def test_pcf_float_loop_is_asymmetric():
    # k = 3: offsets w, h in {-1, -1/3, +1/3} texels -> columns {7, 8, 8}
    S = 16
    s = t = 8.5 / S
    left = np.ones(S * S, np.float32)
    left[8 * S + 7] = 0.1
    right = np.ones(S * S, np.float32)
    right[8 * S + 9] = 0.1
    kw = dict(kernel_order=3, penumbra_size=1)
    assert _probe(api.GI_TECH_PCF, left, S, s, t, 0.5, **kw) == pytest.approx((7 + 2 * 0.25) / 9, abs=1e-7)
    assert _probe(api.GI_TECH_PCF, right, S, s, t, 0.5, **kw) == 1.0


def test_hard_border_is_shadowed_and_background_is_zero():
    S = 8
    m = np.ones(S * S, np.float32)
    assert _probe(api.GI_TECH_HARD, m, S, 0.5, 0.5, 0.5) == 1.0
    assert _probe(api.GI_TECH_HARD, m, S, 1.0, 0.5, 0.5) == 0.25  # s = 1 -> texel S -> border 0
    assert _probe(api.GI_TECH_HARD, m, S, 0.5, -0.01, 0.5) == 0.25
    assert _probe(api.GI_TECH_HARD, m, S, 0.0, 0.5, 0.5) == 0.0  # vertex.x == 0: background


def test_pcss_cutoffs():
    S = 64
    m = np.full(S * S, 0.9, np.float32)  # every blocker at window depth 0.9
    kw = dict(light_radius=2.0, kernel_size=15, blocker_search_size=7)
    # reference cut-off 0.99: average blocker 0.9 < 0.99 -> penumbra 0 -> lit
    assert _probe(api.GI_TECH_PCSS_GRID, m, S, 0.5, 0.5, 0.95, **kw) == 1.0
    assert _probe(api.GI_TECH_PCSS_POISSON, m, S, 0.5, 0.5, 0.95, **kw) == 1.0
    # without the cut-off the receiver is in umbra: every filter tap shadowed
    kw["pcss_min_blocker_depth"] = 0.0
    assert _probe(api.GI_TECH_PCSS_GRID, m, S, 0.5, 0.5, 0.95, **kw) == pytest.approx(0.25)
    assert _probe(api.GI_TECH_PCSS_POISSON, m, S, 0.5, 0.5, 0.95, **kw) == pytest.approx(0.25)
    # no blocker at all -> average 1 -> (z - 1) < 0 -> step <= 0 -> lit
    assert _probe(api.GI_TECH_PCSS_GRID, np.ones(S * S, np.float32), S, 0.5, 0.5, 0.95, **kw) == 1.0


def test_pcss_penumbra_is_fractional_at_an_edge():
    S = 256
    m = np.ones((S, S), np.float32)
    m[:, : S // 2] = 0.5  # blockers on the left half
    kw = dict(light_radius=8.0, kernel_size=15, blocker_search_size=7, pcss_min_blocker_depth=0.0)
    v = _probe(api.GI_TECH_PCSS_GRID, m.reshape(-1), S, 0.5 + 0.5 / S, 0.5, 0.9, **kw)
    assert 0.25 < v < 1.0


def test_rbsm_variants_on_a_straight_edge():
    # a vertical shadow edge: texels x < 8 block (depth 0.1), receiver z 0.5
    S = 16
    m = np.ones((S, S), np.float32)
    m[:, :8] = 0.1
    m = m.reshape(-1)
    kw = dict(max_search=16, kernel_order=3, penumbra_size=1)
    for tech in (api.GI_TECH_SMSR_CONSERVATIVE, api.GI_TECH_SMSR_NONCONSERVATIVE, api.GI_TECH_RPCF_CONSERVATIVE,
                 api.GI_TECH_RPCF_SMSR, api.GI_TECH_RSMSS):
        lit = _probe(tech, m, S, 12.5 / S, 8.5 / S, 0.5, **kw)
        dark = _probe(tech, m, S, 3.5 / S, 8.5 / S, 0.5, **kw)
        assert lit == 1.0, tech
        assert dark == 0.25, tech
        edge = _probe(tech, m, S, 8.5 / S, 8.5 / S, 0.5, **kw)
        assert 0.25 <= edge <= 1.0, tech


def test_pretest_reference_mode_shadows_back_facing_normals():
    S = 8
    m = np.ones(S * S, np.float32)
    p = gi.ShadowParams.defaults(api.GI_TECH_HARD)
    fr = gi.Frame(IDENTITY, IDENTITY, IDENTITY, IDENTITY, np.eye(3, dtype=np.float32).reshape(-1),
                  np.array([0.0, 0.0, 10.0], np.float32))
    pos = np.array([0.5, 0.5, 0.5, 1.0, 0.5, 0.5, 0.5, 1.0, 0.5, 0.5, 0.5, 1.0], np.float32)
    # normal towards the light, away from it, and away but back-facing (flipped)
    nrm = np.array([0, 0, 1, 1, 0, 0, -1, 1, 0, 0, -1, 0], np.float32)
    out = oracle.visibility(p.to_c(fr), m, S, S, pos, nrm, 3, 1)
    assert out.tolist() == [1.0, 0.25, 1.0]


def test_shadow_volume_counts_match_a_ray_test():
    # one occluder triangle above a ground quad; pixels far from the shadow
    # boundary must count non-zero exactly when the ground point's segment to
    # the light crosses the triangle (the reference's extrusion (v - L) * 100
    # bends the volume slightly, hence the margin).
    W, H = 96, 72
    s = gi.Scene()
    s.ground(10.0, 0.0)
    s.object_from_arrays(np.array([[-1.5, 2.0, -1.0], [1.5, 2.0, -1.0], [0.0, 2.0, 2.0]], np.float32),
                         [[0, 2, 1]]).commit()
    L = np.array([0.5, 9.0, 0.5], np.float32)
    cam = gi.ViewSpec(eye=(0.0, 12.0, -6.0), at=(0.0, 0.0, 0.0), width=W, height=H)
    fr = gi.frame_setup(gi.ViewSpec(eye=tuple(L), at=(0, 0, 0), width=8, height=8), cam)
    p, n, i = s.arrays()
    st, _ = oracle.shadow_volume_counts(p, n, i, L, 100.0, fr.camera_mvp, W, H, api.GI_DEPTH_LEQUAL)
    pos, _ = oracle.gbuffer(p, n, i, fr.camera_mvp, W, H)
    pos = pos.reshape(H, W, 4)
    st = st.reshape(H, W)
    tri = p[4:7].astype(np.float64)
    checked = 0
    for y in range(H):
        for x in range(W):
            g = pos[y, x, :3].astype(np.float64)
            if pos[y, x, 0] == 0.0 or abs(g[1]) > 1e-4:
                continue  # background or the occluder itself
            # segment g -> L against the plane y = 2 of the triangle
            t = (2.0 - g[1]) / (L[1] - g[1])
            q = g + t * (L - g)
            a, b, c = tri
            d = [np.cross(b - a, q - a)[1], np.cross(c - b, q - b)[1], np.cross(a - c, q - c)[1]]
            margin = 0.15
            dist = min(abs(v) / np.linalg.norm(e) for v, e in zip(d, (b - a, c - b, a - c)))
            if dist < margin:
                continue
            inside = all(v > 0 for v in d) or all(v < 0 for v in d)
            assert (st[y, x] != 0) == inside, (x, y, st[y, x])
            checked += 1
    assert checked > 2000
    assert (st != 0).sum() > 100


def _rbssm_kw(**extra):
    kw = dict(light_radius=8.0, kernel_size=7, blocker_search_size=7, max_search=16, depth_threshold=0.0,
              pcss_min_blocker_depth=0.0)
    kw.update(extra)
    return kw


def test_rbssm_lit_and_umbra():
    S = 64
    # no blocker anywhere: average depth 1, negative penumbra, lit
    assert _probe(api.GI_TECH_RBSSM, np.ones(S * S, np.float32), S, 0.5, 0.5, 0.9995, **_rbssm_kw()) == 1.0
    # a uniform blocker plane: every tap is shadowed and none is a discontinuity
    m = np.full(S * S, 0.995, np.float32)
    assert _probe(api.GI_TECH_RBSSM, m, S, 0.5, 0.5, 0.9995, **_rbssm_kw()) == 0.25
    # the reference's 0.99 cut-off on the average blocker depth returns 0 -> lit
    m = np.full(S * S, 0.5, np.float32)
    assert _probe(api.GI_TECH_RBSSM, m, S, 0.5, 0.5, 0.9, **_rbssm_kw(pcss_min_blocker_depth=0.99)) == 1.0


def test_rbssm_straight_edge_known_answer():
    # Vertical edge: texels x < 32 hold blockers at 0.995, the rest is lit.
    # On an axis-aligned edge every discontinuity tap is filled binary:
    # an entering tap (lit, shadowed left neighbour) gets 1, an exiting tap
    # (shadowed, lit right neighbour) gets 0, so the result is the count of
    # lit taps over K^2 with shadowed taps weighted by the intensity 0.25.
    S, z = 64, np.float32(0.999)
    m = np.ones((S, S), np.float32)
    m[:, :32] = 0.995
    s = t = np.float32(32.5 / S)
    kw = _rbssm_kw()
    got = _probe(api.GI_TECH_RBSSM, m.reshape(-1), S, float(s), float(t), float(z), **kw)
    # replay the blocker search and the tap positions in FP32
    f = np.float32
    bsw = f(8.0) / f(S)
    fw = f(3.0)
    total, nb = f(0.0), 0
    for h in range(-3, 4):
        for w in range(-3, 4):
            x = int(np.floor((s + (f(w) * bsw) / fw) * f(S)))
            if x < 32:
                total = f(total + f(0.995))
                nb += 1
    avg = f(total / f(nb))
    pw = f(f(f(z - avg) / avg) * f(8.0))
    pw = f(f(f(1.0) * pw) / z)
    lit = sum(1 for w in range(-3, 4) if int(np.floor((s + (f(w) * pw) / fw) * f(S))) >= 32)
    expect = f(f(7 * (lit * 1.0 + (7 - lit) * 0.25)) / f(49))
    assert 0 < lit < 7
    assert got == float(expect)


def test_rbssm_corner_is_fractional():
    S = 64
    m = np.ones((S, S), np.float32)
    m[:32, :32] = 0.995  # blocker quadrant
    v = _probe(api.GI_TECH_RBSSM, m.reshape(-1), S, 32.5 / S, 32.5 / S, 0.999, **_rbssm_kw())
    assert 0.25 < v < 1.0


def test_rbssm_fuzz_reaches_every_reachable_case():
    # 71 return sites; four cannot be reached: the two "fill all" returns of
    # the both-positive case need nd <= -2 on the axis whose lengths are the
    # early -1 returns, the r == 0.75 exit of the top/bottom case is taken by
    # an earlier case, and the final return needs r == g == 0.
    from rbssm_fuzz import CASES, case

    sites = oracle.rbssm_return_sites()
    assert len(sites) == 71
    oracle.rbssm_hits(reset=True)
    for k in range(len(CASES)):
        p, fr, depth, pos, nrm, S, W, H = case(k)
        v = oracle.visibility(p.to_c(fr), depth, S, S, pos, nrm, W, H)
        assert ((v > 0.25) & (v < 1.0)).mean() > 0.3
    hits = oracle.rbssm_hits()
    covered = [s for s in sites if (s & 4095) in hits]
    assert len(covered) >= len(sites) - 4, sorted(set(sites) - set(covered))


def test_area_light_samples_follow_the_reference_grid():
    light = gi.ViewSpec(eye=(1.0, 12.0, -2.0), at=(0.5, 0.0, 0.25), width=64, height=64, fovy_deg=90.0)
    views = gi.area_light_samples(light, 16.0, 17)
    assert len(views) == 289
    f32 = np.float32
    half, factor = f32(8.0), f32(17.0)
    c = f32((factor - f32(1.0)) / 2.0)
    for i in (0, 1, 16, 17, 144, 288):
        dx = f32(f32(f32(i % 17) - c) / c) * half
        dy = f32(f32(f32(int(f32(i) / factor)) - c) / c) * half
        assert views[i].eye == (float(f32(f32(1.0) + dx)), float(f32(f32(12.0) + dy)), -2.0)
        assert views[i].at == (float(f32(f32(0.5) + dx)), float(f32(f32(0.0) + dy)), 0.25)
    assert views[144].eye == light.eye  # centre sample


def _area_scene(occluder: bool):
    s = gi.Scene()
    s.ground(4.0, 0.0)
    if occluder:
        s.object_from_arrays(np.array([[-1.5, 3.0, -1.5], [1.5, 3.0, -1.5], [1.5, 3.0, 1.5], [-1.5, 3.0, 1.5]],
                                      np.float32), [[0, 2, 1], [0, 3, 2]]).commit()
    return s


def _area_truth(s, n_side=3, S=64, W=48, H=40):
    light = gi.ViewSpec(eye=(0.0, 12.0, 0.0), at=(0.0, 0.0, 0.0), width=S, height=S, fovy_deg=90.0, up=(0, 0, 1))
    cam = gi.ViewSpec(eye=(0.0, 10.0, -1.0), at=(0.0, 0.0, 0.0), width=W, height=H, fovy_deg=40.0)
    views = gi.area_light_samples(light, 1.0, n_side)
    frames = [gi.frame_setup(v, cam) for v in views]
    mvps = np.stack([f.light_mvp for f in frames])
    biased = np.stack([f.light_mvp_biased for f in frames])
    p, n, i = s.arrays()
    v = oracle.area_light_visibility(p, n, i, mvps, biased, S, api.GI_BIAS_POLYGON_OFFSET, 0.0, 4.0, 20.0,
                                     frames[0].camera_mvp, 0.25, W, H)
    pos, _ = oracle.gbuffer(p, n, i, frames[0].camera_mvp, W, H)
    return v, pos.reshape(-1, 4)[:, 0] != 0


def test_area_light_truth_lit_and_umbra():
    v, geo = _area_truth(_area_scene(False))
    assert geo.sum() > 500 and (v[geo] == 1.0).all() and (v[~geo] == 0.0).all()
    v, geo = _area_truth(_area_scene(True))
    # a plate at y = 3 over the ground: umbra below it, penumbra (fractions
    # of the 9 samples) around it, lit ground and plate elsewhere
    g = v[geo]
    assert (g >= 0.25).all() and (g <= 1.0).all()
    assert (g == 0.25).sum() > 10 and (g == 1.0).sum() > 500 and ((g > 0.25) & (g < 1.0)).sum() > 10


def test_phong_single_pixel_known_answer():
    f = np.float32
    p = gi.ShadowParams.defaults(api.GI_TECH_HARD)
    fr = gi.Frame(IDENTITY, IDENTITY, IDENTITY, IDENTITY, np.eye(3, dtype=np.float32).reshape(-1),
                  np.array([0.5, 0.0, 10.0], np.float32))
    pos = np.array([0.5, 0.0, -5.0, 1.0, 0.0, 0.0, 0.0, 1.0], np.float32)  # one surface pixel, one background
    nrm = np.array([0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 0.0, 1.0], np.float32)
    vis = np.array([1.0, 0.0], np.float32)
    out = oracle.phong_shade(p.to_c(fr), pos, nrm, vis, 2, 1).reshape(2, 4)
    # N = L = R = (0, 0, 1); E = (-0.5, 0, 5) / sqrt(26.25) from the 4-component normalise
    e = f(f(5.0) * f(f(1.0) / np.sqrt(f(26.25), dtype=np.float32)))
    spec = f(f(e * e) * e)
    rgb = f(f(f(0.5) + f(f(f(0.75) * f(0.25)) * spec)) + f(0.4))
    alpha = f(f(f(1.0) + f(f(0.75) * spec)) + f(1.0))  # diffuse and ambient alpha are 1
    assert out[0].tolist() == [float(rgb)] * 3 + [float(alpha)]
    assert out[1].tolist() == [float(f(0.63)), float(f(0.82)), float(f(0.96)), 1.0]


def _moment_probe(tech, depth_map, S, s, t, z):
    """Like _probe, but the window is S x S (the moment techniques blur the
    map into a window-size target): pixel 0 carries the probe, the others
    are background."""
    p = gi.ShadowParams.defaults(tech)
    p.pretest = api.GI_PRETEST_OFF
    fr = gi.Frame(IDENTITY, IDENTITY, IDENTITY, IDENTITY, np.eye(3, dtype=np.float32).reshape(-1),
                  np.zeros(3, np.float32))
    pos = np.zeros((S * S, 4), np.float32)
    pos[0] = (s, t, z, 1.0)
    nrm = np.tile(np.array([0, 0, 1, 1], np.float32), (S * S, 1))
    return float(oracle.visibility(p.to_c(fr), depth_map, S, S, pos, nrm, S, S)[0])


@pytest.mark.parametrize("tech", [api.GI_TECH_VSM, api.GI_TECH_ESM, api.GI_TECH_EVSM, api.GI_TECH_MSM])
def test_moment_maps_front_lit_behind_shadowed(tech):
    # a flat blocker at window depth 0.5 over the whole map: a receiver in
    # front of it is lit by every moment technique, one behind it is
    # shadowed (VSM / EVSM / MSM down to about the intensity; ESM, whose
    # exp(80 (m - z)) acts on linearised depths near 0.004, only partly)
    S = 32
    m = np.full(S * S, 0.5, np.float32)
    front = _moment_probe(tech, m, S, 0.5, 0.5, 0.4)
    behind = _moment_probe(tech, m, S, 0.5, 0.5, 0.6)
    assert front == 1.0
    if tech == api.GI_TECH_ESM:
        assert 0.25 <= behind < 0.95
    else:
        assert behind == pytest.approx(0.25, abs=2e-3)


def test_vsm_variance_softens_a_depth_step():
    # two blocker depths side by side: after the 7-tap blur the texels near
    # the step carry variance, and a receiver between the two depths there
    # gets a Chebyshev bound strictly between the intensity and 1
    S = 32
    m = np.full((S, S), 0.45, np.float32)
    m[:, S // 2:] = 0.55
    v = _moment_probe(api.GI_TECH_VSM, m.reshape(-1), S, (S // 2 - 1.5) / S, 0.5, 0.5)
    assert 0.25 < v < 1.0
