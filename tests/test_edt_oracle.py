"""The CPU oracle of the EDT path (PBA distance transform, EDTSM), pinned.

tests/golden/edt_pin.npz holds what the reference's own PBA kernels
(ShadowMapping/include/EDT/pba2DKernel.h, run on the CPU by
oracle/ref_pba_pin.cpp) produce for the cases of tests/edt_cases.py; the
oracle must reproduce it bit for bit, equidistant sites included.  Where the
reference tree is present the oracle is also compared live with those
kernels on further seeded inputs.  Distances are checked against brute
force.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from edt_cases import EDT_CASES, MARKER, PBA_CASES, brute_force_sqdist, hard_shadow_image, pba_case, site_mask, \
    sites_from_mask

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "edt_pin.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def ref_lib():
    from oracle.build_oracle import build_pba_ref

    path = build_pba_ref()
    if path is None:
        pytest.skip("the reference's PBA kernels are not available here")
    return C.CDLL(path)


def _sqdist(nearest):
    H, W = nearest.shape[:2]
    yy, xx = np.mgrid[0:H, 0:W]
    return (nearest[..., 0].astype(np.int64) - xx) ** 2 + (nearest[..., 1].astype(np.int64) - yy) ** 2


@pytest.mark.parametrize("case", [c[0] for c in PBA_CASES])
def test_pba_oracle_matches_reference_golden(golden, case):
    sites, bands = pba_case(case)
    got = oracle.pba_voronoi(sites, bands)
    np.testing.assert_array_equal(got, golden[f"pba/{case}/nearest"])


@pytest.mark.parametrize("case", [c[0] for c in PBA_CASES if c[3] != "empty"])
def test_pba_oracle_is_exact(case):
    sites, bands = pba_case(case)
    m = sites[..., 0] != MARKER
    got = oracle.pba_voronoi(sites, bands)
    assert m[got[..., 1], got[..., 0]].all(), "every pixel must point at a site"
    np.testing.assert_array_equal(_sqdist(got), brute_force_sqdist(m))


def test_pba_empty_image_points_at_minus_one_zero():
    # the reference's coloring reads outside its texture for a line without
    # sites (tex1Dfetch returns 0 there), which yields site (-1, 0)
    sites = sites_from_mask(np.zeros((64, 64), bool))
    got = oracle.pba_voronoi(sites)
    assert (got[..., 0] == -1).all() and (got[..., 1] == 0).all()


@pytest.mark.parametrize("case", [c[0] for c in EDT_CASES])
def test_edtsm_oracle_matches_reference_golden(golden, case):
    name, W, H, seed, pen, inten, bands = next(c for c in EDT_CASES if c[0] == case)
    img, pos = hard_shadow_image(W, H, seed)
    out4, sites, nearest = oracle.edt_soft_shadows(img, pos, np.float32(pen / 5.0), inten, bands)
    np.testing.assert_array_equal(sites, golden[f"edt/{case}/sites"])
    np.testing.assert_array_equal(nearest, golden[f"edt/{case}/nearest"])
    np.testing.assert_array_equal(out4[..., :2].view(np.uint32), golden[f"edt/{case}/out01"].view(np.uint32))


def test_edtsm_golden_cases_exercise_every_branch(golden):
    # umbra and lit pixels inside the penumbra, and pixels left at their hard value
    changed_umbra = changed_lit = kept = 0
    for name, W, H, seed, *_ in EDT_CASES:
        img, _ = hard_shadow_image(W, H, seed)
        out = golden[f"edt/{name}/out01"][..., 0]
        diff = out != img[..., 0]
        changed_umbra += int((diff & (img[..., 0] == 0.25)).sum())
        changed_lit += int((diff & (img[..., 0] == 1.0)).sum())
        kept += int((~diff & (img[..., 2] == 1.0)).sum())
    assert changed_umbra > 50 and changed_lit > 50 and kept > 1000


def _ref_pba(lib, sites, bands):
    H, W = sites.shape[:2]
    out = np.empty_like(sites)
    assert lib.ref_pba_voronoi(sites.ctypes.data_as(C.c_void_p), W, H, *bands,
                               out.ctypes.data_as(C.c_void_p)) == 0
    return out


@pytest.mark.parametrize("W", [64, 128, 256])
@pytest.mark.parametrize("bands", [(16, 16, 16), (4, 8, 4), (32, 2, 1), (2, 32, 64)])
def test_pba_oracle_matches_reference_kernels_live(ref_lib, W, bands):
    if W // bands[0] < 2 or W // bands[1] < 2:
        pytest.skip("bands of one row / pixel are outside the supported shapes")
    for seed, (kind, p) in enumerate([("random", 0.003), ("random", 0.05), ("lattice", 7), ("lines", 4),
                                      ("clusters", 6)]):
        sites = sites_from_mask(site_mask(kind, W, W, p, 100 + seed))
        np.testing.assert_array_equal(oracle.pba_voronoi(sites, bands), _ref_pba(ref_lib, sites, bands),
                                      err_msg=f"{kind} {p}")


def test_edtsm_oracle_matches_reference_kernels_live(ref_lib):
    for seed in range(4):
        W = 64 * (1 + seed % 2)
        img, pos = hard_shadow_image(W, W, 300 + seed)
        out4 = np.zeros((W, W, 4), np.float32)
        nn = np.empty((W, W, 2), np.int16)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        assert ref_lib.ref_edt_soft_shadows(vp(img), vp(pos), W, W, 16, 16, 16, C.c_float(0.6), C.c_float(0.25),
                                            None, vp(nn), vp(out4)) == 0
        got, _, gnn = oracle.edt_soft_shadows(img, pos, np.float32(0.6), 0.25)
        np.testing.assert_array_equal(gnn, nn)
        np.testing.assert_array_equal(got[..., :2].view(np.uint32), out4[..., :2].view(np.uint32))


def _lin(d):
    # linearize (pba2DKernel.h:499-506): float denominator, double division
    den = np.float32(1001.0) - np.float32(d) * np.float32(999.0)
    return np.float32(2.0 / np.float64(den))


def threshold_depths(a=np.float32(0.5)):
    """Depths b_in, b_out next to each other with |lin(a) - lin(b)| <= 0.0025 for b_in only."""
    lo, hi = np.float32(a).view(np.int32), np.float32(0.99).view(np.int32)
    passes = lambda b: float(abs(np.float32(_lin(a) - _lin(b)))) <= 0.0025  # noqa: E731
    assert passes(np.int32(lo).view(np.float32)) and not passes(np.int32(hi).view(np.float32))
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if passes(np.int32(mid).view(np.float32)):
            lo = mid
        else:
            hi = mid
    return np.int32(lo).view(np.float32), np.int32(hi).view(np.float32)


def threshold_image(b, a=np.float32(0.5)):
    img = np.zeros((8, 8, 4), np.float32)
    img[..., 2:] = 1.0
    img[:, :4, 0], img[:, :4, 1] = 1.0, a
    img[:, 4:, 0], img[:, 4:, 1] = 0.25, b
    return img


def test_site_threshold_is_the_references_double_comparison():
    # initializeInput compares the float |linearize(a) - linearize(b)| with
    # the double literal 0.0025: depths one float apart straddle it
    b_in, b_out = threshold_depths()
    s_in = oracle.edt_sites(threshold_image(b_in))
    s_out = oracle.edt_sites(threshold_image(b_out))
    assert (s_in[:, 3:5, 0] != MARKER).all() and (s_in[:, :3, 0] == MARKER).all()
    assert (s_out[..., 0] == MARKER).all()


def test_mean_filter_known_answers():
    # 32 x 32 geometry at eye depth 50 (identity MV, vertex z = -50): the
    # half-width is 50 * 7 / (2 tan(22.5) * 2 * 50) = 3.13 samples, so 7
    # samples per pass.  A 0.25 / 1.0 step at one depth is averaged across
    # the step, a region at another depth is left alone, background keeps
    # (0, 0, 0, 1).
    import globalillumination_gb300 as gi
    from globalillumination_gb300 import _capi as api

    W = H = 32
    p = gi.ShadowParams.defaults(api.GI_TECH_SMSR_NONCONSERVATIVE)
    fr = gi.Frame(*(np.eye(4, dtype=np.float32).reshape(-1),) * 4, np.eye(3, dtype=np.float32).reshape(-1),
                  np.zeros(3, np.float32))
    pos = np.zeros((H, W, 4), np.float32)
    pos[...] = (1.0, 1.0, -50.0, 1.0)
    pos[0, 0, 0] = 0.0  # one background pixel
    img = np.zeros((H, W, 4), np.float32)
    img[..., 0] = np.where(np.arange(W) < W // 2, 0.25, 1.0)[None, :]
    img[..., 1] = 0.98
    img[:, 28:, 1] = 0.5  # a region far in front: its own depth class
    out = oracle.edt_mean_filter(p.to_c(fr), img, pos, W, H)
    assert tuple(out[0, 0]) == (0.0, 0.0, 0.0, 1.0)
    assert out[10, 5, 0] == pytest.approx(0.25) and out[10, 5, 1] == np.float32(0.98)
    row = out[10, :, 0]
    assert 0.25 < row[W // 2 - 1] < row[W // 2] < 1.0  # the step is smoothed over about 3 texels
    assert row[W // 2 - 5] == pytest.approx(0.25) and row[W // 2 + 4] == pytest.approx(1.0)
    # depth 0.5 pixels only average among themselves (away from the top and
    # bottom rows, where the bilinear y pass blends in the zero border)
    assert (out[5:27, 28:, 0] == 1.0).all()
