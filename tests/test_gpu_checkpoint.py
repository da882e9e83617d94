"""Resuming surrogate training from a checkpoint is bit-identical.

Twelve Adam steps in one run against six steps, a checkpoint (weights,
biases, Adam moments and step of every layer, the next step, the data RNG),
a fresh network and trainer loading it, and six more steps: the losses of
the last six steps and every final weight agree bit for bit (the training
kernels reduce gradients in a fixed order)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from globalillumination_gb300 import surrogate as sg  # noqa: E402

pytestmark = pytest.mark.gpu


def test_resumed_training_is_bit_identical(cuda_ctx, tmp_path):
    kw = dict(batch=4, crop=128, lr=1e-3, scenes_in_pool=3, seed=0x5EED0077)
    full = sg.Trainer(cuda_ctx, sg.UNet(0, seed=3), **kw)
    h_full = full.run(12, log_every=1, verbose=False)
    first = sg.Trainer(cuda_ctx, sg.UNet(0, seed=3), **kw)
    first.run(6, log_every=1, verbose=False)
    path = os.path.join(str(tmp_path), "ckpt.npz")
    first.save(path)
    second = sg.Trainer(cuda_ctx, sg.UNet(0, seed=99), **kw)  # different init: everything comes from the file
    second.load(path)
    assert second.step == 6
    h_res = second.run(6, log_every=1, verbose=False)
    assert [h["step"] for h in h_res] == list(range(7, 13))
    for a, b in zip(h_full[6:], h_res):
        assert a["step"] == b["step"]
        assert np.float32(a["mae"]).view(np.uint32) == np.float32(b["mae"]).view(np.uint32), (a, b)
        assert np.float32(a["err_l1"]).view(np.uint32) == np.float32(b["err_l1"]).view(np.uint32), (a, b)
    sa, sb = sg.net_full_state(full.net), sg.net_full_state(second.net)
    for k in sa:
        assert np.array_equal(np.asarray(sa[k]).reshape(-1).view(np.uint8), np.asarray(sb[k]).reshape(-1).view(np.uint8)), k
    assert full.net.kernel_error() == 0 and second.net.kernel_error() == 0
