"""oracle/pcss_1080p_inputs.npz (the CPU baseline's inputs) equals what the
product's generators make for the pcss_1080p workload, bit for bit, so the
two arms of bench.py render the same frame."""
import numpy as np

from oracle.bench_inputs import Inputs, make


def test_archive_equals_product_workload():
    fresh = make(path=None)
    inp = Inputs()
    for name in ("points", "normals", "indices", "light_mvp", "camera_mvp", "poisson"):
        a, b = np.asarray(fresh[name]), getattr(inp, name)
        assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), name
    assert bytes(inp.vis_params) == fresh["vis_params"].tobytes()
    assert [inp.S, inp.bias_mode] == fresh["map"].tolist()
    assert [inp.W, inp.H] == fresh["camera"].tolist()
    assert np.array_equal(np.array([inp.constant_bias, inp.offset_factor, inp.offset_units], np.float32),
                          fresh["map_bias"])
