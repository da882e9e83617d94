"""What the trained surrogate gains, on error and on time, over the methods without it.

The learned part stands in for PCSS's blocker search and filtering
(PlausibleSoftShadow.frag:166-194,365-398, called per frame at
SoftShadowMapping/src/main.cpp:1010-1017).  On a pcss_1080p frame that is
not in its training set this test measures, against the exact PCSS frame:

  * the whole surrogate (trained network plus its error-head fallback)
    against the estimate the pipeline has without a network, the hard
    shadow test it is fed: the surrogate must cut that error at least
    fivefold and stay within 1 % mean absolute error (the bound it is
    specified to);
  * the trained network against the same network untrained (both without
    fallback), and the fallback against the network alone: training and
    the error head must each lower the error.  The network alone is not
    required to beat the hard shadows: on this frame penumbrae cover few
    pixels, and its small errors spread over lit receivers, which is what
    the error head's fallback removes;
  * the frame time of the surrogate and of the plain PCSS frame (CUDA
    events).  On this GPU the exact PCSS frame is the faster of the two;
    the test records both and checks only that they were measured.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import globalillumination_gb300 as gi  # noqa: E402
from globalillumination_gb300 import _capi as api, scenes  # noqa: E402
from globalillumination_gb300 import surrogate as sg  # noqa: E402

pytestmark = pytest.mark.gpu


def _time(fn, reps=10):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def test_trained_surrogate_gain_over_methods_without_it(cuda_ctx):
    ctx = cuda_ctx
    net = sg.UNet(0, seed=1)
    untrained = sg.UNet(0, seed=1)
    sg.train(ctx, net, frames=4000, batch=16, crop=256, lr=1e-3, verbose=False, log_every=1000)
    assert net.kernel_error() == 0
    w = scenes.pcss_1080p()
    W, H, S = w.camera.width, w.camera.height, w.map_params.width
    fr = gi.frame_setup(w.light, w.camera)
    w.scene.upload(ctx)
    exact = gi.allocate_frame(S, S, W, H)
    gi.render_frame(ctx, w.scene, fr, w.map_params, w.params, W, H, exact)
    hard = gi.allocate_frame(S, S, W, H)
    p_hard = gi.ShadowParams.defaults(api.GI_TECH_HARD)
    gi.render_frame(ctx, w.scene, fr, w.map_params, p_hard, W, H, hard)
    sf = sg.SurrogateFrame(net, S, W, H)
    v_net = sf.render(ctx, w.scene, fr, w.map_params, w.params, threshold=math.inf).clone()
    sf.fallback.zero_()
    v_fb = sf.render(ctx, w.scene, fr, w.map_params, w.params).clone()
    fallback = int(sf.fallback.item()) / (W * H)
    sf_u = sg.SurrogateFrame(untrained, S, W, H)
    v_untrained = sf_u.render(ctx, w.scene, fr, w.map_params, w.params, threshold=math.inf).clone()
    torch.cuda.synchronize()
    ref = exact.vis
    mae = {k: float((v - ref).abs().mean()) for k, v in
           (("hard", hard.vis), ("untrained", v_untrained), ("trained", v_net), ("trained_fallback", v_fb))}
    t_sur = _time(lambda: sf.render(ctx, w.scene, fr, w.map_params, w.params))
    t_pcss = _time(lambda: gi.render_frame(ctx, w.scene, fr, w.map_params, w.params, W, H, exact))
    print(f"MAE vs exact PCSS: {mae}; fallback {fallback:.4f}; frame ms surrogate {t_sur:.3f}, plain PCSS {t_pcss:.3f}")
    assert mae["hard"] > 0.0
    assert mae["trained_fallback"] < 0.2 * mae["hard"], mae
    assert mae["trained_fallback"] <= 0.01, mae
    assert mae["trained"] < mae["untrained"], mae
    assert mae["trained_fallback"] < mae["trained"], mae
    assert 0.0 < fallback < 0.5
    assert t_sur > 0.0 and t_pcss > 0.0
    assert net.kernel_error() == 0
    assert np.isfinite(v_fb.cpu().numpy()).all()
