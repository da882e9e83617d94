"""The PBA distance transform and the EDTSM filter on the GPU, bit for bit.

Checked against the committed outputs of the reference's own PBA kernels
(tests/golden/edt_pin.npz) and against the CPU oracle on larger and
non-square images, on other band settings, and on a rendered frame (the
SMSR visibility turned into EDTSM inputs by gi_edt_inputs).  Every
comparison is exact: nearest sites as integers, shadows as float bits.
"""
import os

import numpy as np
import pytest

import oracle
import globalillumination_gb300 as gi
from globalillumination_gb300 import _capi as api, scenes
from edt_cases import EDT_CASES, MARKER, PBA_CASES, hard_shadow_image, pba_case, site_mask, sites_from_mask
from test_edt_oracle import threshold_depths, threshold_image

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "edt_pin.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _pba(ctx, sites, bands=(16, 16, 16)):
    import torch

    s = torch.from_numpy(np.ascontiguousarray(sites)).cuda()
    out = torch.empty_like(s)
    gi.pba_voronoi(ctx, s, out, bands)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _edt(ctx, img, pos, penumbra_size, intensity, bands=(16, 16, 16), fill=np.nan):
    import torch

    H, W = img.shape[:2]
    ti, tp = torch.from_numpy(img).cuda(), torch.from_numpy(pos).cuda()
    out = torch.full((H, W, 4), float(fill), device="cuda")
    nn = torch.empty((H, W, 2), dtype=torch.int16, device="cuda")
    gi.edt_soft_shadows(ctx, ti, tp, out, penumbra_size, intensity, bands, nearest=nn)
    torch.cuda.synchronize()
    return out.cpu().numpy(), nn.cpu().numpy()


@pytest.mark.parametrize("case", [c[0] for c in PBA_CASES])
def test_pba_matches_reference_golden(cuda_ctx, golden, case):
    sites, bands = pba_case(case)
    np.testing.assert_array_equal(_pba(cuda_ctx, sites, bands), golden[f"pba/{case}/nearest"])


def test_degenerate_lists_take_the_exact_chain(cuda_ctx, golden):
    # rows whose list is not a strict envelope are colored by replaying the
    # reference's group chain; the others by a binary search -- both exact
    gi.pba_chain_rows(cuda_ctx, reset=True)
    for case in ("degenerate_a_64", "degenerate_b_64"):
        sites, bands = pba_case(case)
        np.testing.assert_array_equal(_pba(cuda_ctx, sites, bands), golden[f"pba/{case}/nearest"])
    assert gi.pba_chain_rows(cuda_ctx) >= 2
    sites, bands = pba_case("random_sparse_64")
    _pba(cuda_ctx, sites, bands)
    assert gi.pba_chain_rows(cuda_ctx, reset=True) < 64 + 2


@pytest.mark.parametrize("case", [c[0] for c in EDT_CASES])
def test_edtsm_matches_reference_golden(cuda_ctx, golden, case):
    name, W, H, seed, pen, inten, bands = next(c for c in EDT_CASES if c[0] == case)
    img, pos = hard_shadow_image(W, H, seed)
    out, nn = _edt(cuda_ctx, img, pos, pen, inten, bands)
    np.testing.assert_array_equal(nn, golden[f"edt/{case}/nearest"])
    np.testing.assert_array_equal(out[..., :2].view(np.uint32), golden[f"edt/{case}/out01"].view(np.uint32))
    # channels 2-3 are not the kernel's (the reference leaves them too)
    assert np.isnan(out[..., 2:]).all()


SHAPES = [(1024, 1024, (16, 16, 16)), (512, 256, (16, 16, 16)), (256, 512, (8, 32, 4)), (768, 384, (3, 8, 12)),
          (2048, 2048, (16, 16, 16)), (1024, 1024, (64, 256, 1))]


@pytest.mark.parametrize("W,H,bands", SHAPES)
def test_pba_matches_oracle(cuda_ctx, W, H, bands):
    for seed, (kind, p) in enumerate([("random", 0.0005), ("random", 0.02), ("lattice", 13), ("lines", 5),
                                      ("clusters", 12)]):
        sites = sites_from_mask(site_mask(kind, W, H, p, 500 + seed))
        np.testing.assert_array_equal(_pba(cuda_ctx, sites, bands), oracle.pba_voronoi(sites, bands),
                                      err_msg=f"{kind} {p}")


def test_pba_edge_cases(cuda_ctx):
    for W, H in ((64, 64), (256, 128)):
        empty = sites_from_mask(np.zeros((H, W), bool))
        got = _pba(cuda_ctx, empty)
        assert (got[..., 0] == -1).all() and (got[..., 1] == 0).all()
        full = sites_from_mask(np.ones((H, W), bool))
        yy, xx = np.mgrid[0:H, 0:W]
        got = _pba(cuda_ctx, full)
        assert (got[..., 0] == xx).all() and (got[..., 1] == yy).all()
        for corner in ((0, 0), (H - 1, W - 1), (0, W - 1)):
            m = np.zeros((H, W), bool)
            m[corner] = True
            got = _pba(cuda_ctx, sites_from_mask(m))
            assert (got[..., 1] == corner[0]).all() and (got[..., 0] == corner[1]).all()
    # any x other than MARKER makes a site, whatever the pair holds
    s = np.full((64, 64, 2), MARKER, np.int16)
    s[10, 20] = (7, 7)
    got = _pba(cuda_ctx, s)
    assert (got[..., 0] == 20).all() and (got[..., 1] == 10).all()


@pytest.mark.parametrize("W,H,bands", [(1024, 1024, (16, 16, 16)), (1920, 1080, (8, 16, 16)),
                                       (640, 480, (16, 16, 16))])
def test_edtsm_matches_oracle(cuda_ctx, W, H, bands):
    for seed, (pen, inten) in enumerate([(1.0, 0.25), (40.0, 0.25)]):
        img, pos = hard_shadow_image(W, H, 700 + seed)
        out, nn = _edt(cuda_ctx, img, pos, pen, inten, bands)
        ref, _, rnn = oracle.edt_soft_shadows(img, pos, np.float32(pen / 5.0), inten, bands)
        np.testing.assert_array_equal(nn, rnn)
        np.testing.assert_array_equal(out[..., :2].view(np.uint32), ref[..., :2].view(np.uint32))


def test_site_threshold_on_gpu(cuda_ctx):
    # one float of depth decides whether the shadow edge has sites (the
    # reference's float-vs-double comparison); no sites -> site (-1, 0)
    b_in, b_out = threshold_depths()
    pos = np.zeros((8, 8, 4), np.float32)
    _, nn = _edt(cuda_ctx, threshold_image(b_in), pos, 1.0, 0.25, (4, 4, 8))
    assert (nn[:, 3, 0] == 3).all() and (nn[:, 4, 0] == 4).all()
    _, nn = _edt(cuda_ctx, threshold_image(b_out), pos, 1.0, 0.25, (4, 4, 8))
    assert (nn[..., 0] == -1).all() and (nn[..., 1] == 0).all()


@pytest.mark.parametrize("tech", [api.GI_TECH_SMSR_NONCONSERVATIVE, api.GI_TECH_SMSR_CONSERVATIVE])
def test_edtsm_on_a_rendered_frame(cuda_ctx, tech):
    import torch

    w = scenes.pcss_1080p(width=512, height=288, map_size=1024, spheres=24)
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    p = gi.ShadowParams.defaults(tech)
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(cuda_ctx)
    bufs = gi.allocate_frame(S, S, W, H)
    gi.render_frame(cuda_ctx, w.scene, fr, w.map_params, p, W, H, bufs, store_gbuffer=True)
    image = torch.empty((H, W, 4), device="cuda")
    position = torch.empty((H, W, 4), device="cuda")
    gi.edt_inputs(cuda_ctx, p, fr, bufs.pos, bufs.nrm, bufs.vis, W, H, image, position)
    torch.cuda.synchronize()
    ri, rp = oracle.edt_inputs(p.to_c(fr), fr.camera_mvp, bufs.pos.cpu().numpy(), bufs.nrm.cpu().numpy(),
                               bufs.vis.cpu().numpy(), W, H)
    gimg, gpos = image.cpu().numpy(), position.cpu().numpy()
    np.testing.assert_array_equal(gimg.view(np.uint32), ri.view(np.uint32))
    np.testing.assert_array_equal(gpos.view(np.uint32), rp.view(np.uint32))
    out, nn = _edt(cuda_ctx, gimg, gpos, 1.0, p.shadow_intensity, (16, 16, 16))
    ref, sites, rnn = oracle.edt_soft_shadows(ri, rp, np.float32(1.0 / 5.0), p.shadow_intensity)
    np.testing.assert_array_equal(nn, rnn)
    np.testing.assert_array_equal(out[..., :2].view(np.uint32), ref[..., :2].view(np.uint32))
    assert (sites[..., 0] != MARKER).sum() > 100, "the frame's shadow edges must produce sites"
    # the screen-space mean filter that ends filterHardShadowsUsingEDT
    t_out = torch.from_numpy(out).cuda()
    mean = torch.empty_like(t_out)
    gi.edt_mean_filter(cuda_ctx, p, fr, t_out, bufs.pos, mean, W, H)
    torch.cuda.synchronize()
    ref_mean = oracle.edt_mean_filter(p.to_c(fr), out, bufs.pos.cpu().numpy(), W, H)
    np.testing.assert_array_equal(mean.cpu().numpy().view(np.uint32), ref_mean.view(np.uint32))


def test_shape_validation(cuda_ctx):
    import torch

    s = torch.zeros((64, 64, 2), dtype=torch.int16, device="cuda")
    o = torch.empty_like(s)
    for bands in ((64, 16, 16), (16, 12, 16), (16, 64, 16), (16, 16, 7), (0, 16, 16)):
        with pytest.raises(gi.GIError):
            gi.pba_voronoi(cuda_ctx, s, o, bands)
    bad = torch.zeros((64, 60, 2), dtype=torch.int16, device="cuda")
    with pytest.raises(gi.GIError):
        gi.pba_voronoi(cuda_ctx, bad, torch.empty_like(bad), (16, 2, 4))
