"""The C++ oracle's depth-map rasteriser against a brute-force numpy
restatement of the same rules (tests/raster_ref.py), bit for bit: light maps
of a sphere field in the three bias modes, square and non-square, and a
low camera whose view clips the ground against the near plane."""
import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api

import raster_ref as ref


@pytest.fixture(scope="module")
def scene_arrays():
    s = gi.Scene()
    s.ground(10.0, 0.0)
    s.icosphere_field(8, 2, (-8.0, 0.2, -8.0), (8.0, 3.0, 8.0), 0.4, 1.6, 0x5EED0007)
    arrays = s.arrays()
    s.close()
    return arrays


@pytest.fixture(scope="module")
def mesh(scene_arrays):
    p, _, i = scene_arrays
    return p, i


def _mvp(eye, at, W, H, fovy=90.0):
    v = gi.ViewSpec(eye=eye, at=at, width=W, height=H, fovy_deg=fovy)
    return gi.frame_setup(v, v).light_mvp


CASES = [
    ("light 96^2, no bias", (0.0, 12.0, 0.0), 96, 96, api.GI_BIAS_NONE, {}),
    ("light 96^2, constant bias", (0.0, 12.0, 0.0), 96, 96, api.GI_BIAS_CONSTANT, {"constant_bias": 0.002}),
    ("light 96^2, polygon offset", (0.0, 12.0, 0.0), 96, 96, api.GI_BIAS_POLYGON_OFFSET,
     {"factor": 4.0, "units": 20.0}),
    ("oblique light 80x52, polygon offset", (7.0, 6.0, -5.0), 80, 52, api.GI_BIAS_POLYGON_OFFSET,
     {"factor": 1.5, "units": 4.0}),
    ("low eye over the ground (near-plane clipping)", (0.0, 0.6, -9.5), 72, 40, api.GI_BIAS_NONE, {}),
]


@pytest.mark.parametrize("name,eye,W,H,bias,kw", CASES, ids=[c[0] for c in CASES])
def test_oracle_depth_map_equals_brute_force_restatement(mesh, name, eye, W, H, bias, kw):
    p, i = mesh
    mvp = _mvp(eye, (0.0, 0.0, 0.0), W, H)
    kw_o = dict(constant_bias=kw.get("constant_bias", 0.0), factor=kw.get("factor", 0.0), units=kw.get("units", 0.0))
    got = oracle.shadow_map(p, i, mvp, W, H, bias, **kw_o)
    want = ref.shadow_map(p, i, mvp, W, H, bias, **kw_o)
    diff = got.view(np.uint32) != want.view(np.uint32)
    assert not diff.any(), f"{name}: {int(diff.sum())} of {W * H} texels differ"
    assert (want < 1.0).mean() > 0.2, "the mesh covers the map"


def test_low_eye_case_clips_triangles(mesh):
    """The near-plane case above does exercise clipping: some triangles cross
    z = -w and are cut into polygons of four or more vertices."""
    p, i = mesh
    m = [np.float32(v) for v in _mvp((0.0, 0.6, -9.5), (0.0, 0.0, 0.0), 72, 40).reshape(16)]
    sizes = [len(ref.clip([ref.transform(m, p[k]) for k in t])) for t in i]
    assert any(n >= 4 for n in sizes) and any(n == 0 for n in sizes)


def test_edges_through_pixel_centres_follow_the_top_left_rule():
    """Triangles whose edges pass exactly through pixel centres: which of two
    triangles (at different depths) owns a shared edge's pixels, and which
    outer edges cover their pixels, is the top-left rule's decision."""
    W = H = 16
    ident = np.eye(4, dtype=np.float32).reshape(16)

    def ndc(xw, yw, zw):  # window coordinates -> clip (w = 1) under the identity MVP
        return [(xw - W / 2) / (W / 2), (yw - H / 2) / (H / 2), 2.0 * zw - 1.0]

    pts = np.array([ndc(2.5, 2.5, 0.3), ndc(12.5, 2.5, 0.3), ndc(2.5, 12.5, 0.3),
                    ndc(12.5, 2.5, 0.6), ndc(12.5, 12.5, 0.6), ndc(2.5, 12.5, 0.6),
                    ndc(5.5, 5.5, 0.2), ndc(9.5, 5.5, 0.2), ndc(9.5, 9.5, 0.2)], np.float32)
    idx = np.array([[0, 1, 2], [3, 4, 5], [6, 8, 7]], np.int32)  # the last one clockwise
    got = oracle.shadow_map(pts, idx, ident, W, H)
    want = ref.shadow_map(pts, idx, ident, W, H)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    d = want.reshape(H, W)
    # with y up, the left (x = 2.5) and top (y = 12.5) edges own the pixel
    # centres on them and the right (x = 12.5) and bottom (y = 2.5) ones do
    # not: columns 2..11 and rows 3..12 are covered
    assert (d[3:13, 2:12] < 1).all()
    assert (d[:3, :] == 1).all() and (d[13:, :] == 1).all() and (d[:, :2] == 1).all() and (d[:, 12:] == 1).all()
    # the shared diagonal's pixel centres belong to one triangle only
    za, zb = d[4, 3], d[11, 10]  # inside the first / the second triangle only
    diag = [(y, x) for y in range(3, 13) for x in range(2, 12) if x + y == 14 and not (5 <= x <= 9 and 5 <= y <= 9)]
    assert za != zb and all(d[y, x] in (za, zb) for y, x in diag)


@pytest.mark.parametrize("eye,W,H", [((0.0, 14.0, -20.0), 96, 54), ((0.0, 0.6, -9.5), 72, 40),
                                     ((-9.0, 3.0, 6.0), 64, 64), ((2.0, -6.0, -9.0), 64, 48)],
                         ids=["camera over the field", "low eye (near-plane clipping)", "oblique",
                              "below the ground (back faces)"])
def test_oracle_gbuffer_equals_brute_force_restatement(scene_arrays, eye, W, H):
    """The G-buffer: nearest fragment, first in draw order among equal depths,
    position and normal interpolated perspective-correct (through the
    clipped sub-triangle's source weights), front-facing flag in nrm.w."""
    p, n, i = scene_arrays
    v = gi.ViewSpec(eye=eye, at=(0.0, 0.0, 0.0), width=W, height=H)
    mvp = gi.frame_setup(v, v).camera_mvp
    got_p, got_n = oracle.gbuffer(p, n, i, mvp, W, H)
    want_p, want_n = ref.gbuffer(p, n, i, mvp, W, H)
    assert np.array_equal(got_p.view(np.uint32), want_p.view(np.uint32))
    assert np.array_equal(got_n.view(np.uint32), want_n.view(np.uint32))
    fg = want_p.reshape(-1, 4)[:, 0] != 0
    assert fg.mean() > 0.3
    w = want_n.reshape(-1, 4)[fg, 3]
    if eye[1] < 0:  # the ground seen from below shows its back face
        assert (w == 0.0).any() and (w == 1.0).any()
    else:
        assert (w == 1.0).any()


@pytest.mark.parametrize("func", [api.GI_DEPTH_LESS, api.GI_DEPTH_LEQUAL], ids=["LESS", "LEQUAL"])
def test_oracle_stencil_counts_equal_brute_force_restatement(scene_arrays, func):
    """Shadow-volume stencil counts: the volume triangles are ShadowVolume::
    build's (the oracle's geometry, itself pinned to the reference's own
    code), drawn by the brute-force rasteriser against its own prepass."""
    p, n, i = scene_arrays
    W, H = 80, 48
    v = gi.ViewSpec(eye=(0.0, 9.0, -14.0), at=(0.0, 0.5, 0.0), width=W, height=H)
    mvp = gi.frame_setup(v, v).camera_mvp
    L = np.array([3.0, 12.0, -2.0], np.float32)
    got_st, got_d = oracle.shadow_volume_counts(p, n, i, L, 100.0, mvp, W, H, func)
    vols = oracle.shadow_volume_geometry(p, n, i, L, 100.0)
    want_st, want_d = ref.stencil_counts(p, i, vols, mvp, W, H, func == api.GI_DEPTH_LEQUAL)
    assert np.array_equal(got_d.view(np.uint32), want_d.view(np.uint32))
    assert np.array_equal(got_st, want_st), f"{int((got_st != want_st).sum())} pixels differ"
    assert (want_st != 0).any() and (want_st == 0).any()  # shadowed and lit pixels
