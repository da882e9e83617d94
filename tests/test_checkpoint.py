"""Training checkpoints on the CPU: the archive round-trips every array and
the trainer's position exactly, and the data RNG restored from it draws the
same crops as the original run would have."""
import io

import numpy as np
import pytest

from globalillumination_gb300 import surrogate as sg


def _fake_net_state(rng):
    st = {"step_count": np.array(7, np.int64)}
    for n, _, ci, co, k in sg.ARCH[:3]:
        for key, shape in ((".w", (co, ci, k, k)), (".b", (co,)), (".mw", (co, ci, k, k)), (".mb", (co,)),
                           (".vw", (co, ci, k, k)), (".vb", (co,))):
            st[n + key] = rng.standard_normal(shape).astype(np.float32)
    return st


def test_checkpoint_round_trip_and_rng_resume():
    rng = np.random.default_rng(0x5EED0003)
    rng.random(1000)  # advance: the saved state is mid-run
    trainer_state = {"step": 12, "rng": rng.bit_generator.state, "batch": 16, "crop": 256, "lr": 1e-3,
                     "scenes_in_pool": 24, "seed": 0x5EED0003}
    net_state = _fake_net_state(np.random.default_rng(1))
    buf = io.BytesIO()
    np.savez(buf, **sg.pack_checkpoint(net_state, trainer_state))
    buf.seek(0)
    with np.load(buf) as z:
        got_net, got_tr = sg.unpack_checkpoint(z)
    assert set(got_net) == set(net_state)
    for k, v in net_state.items():
        assert got_net[k].dtype == v.dtype and np.array_equal(got_net[k].reshape(-1).view(np.uint8), v.reshape(-1).view(np.uint8)), k
    assert got_tr == trainer_state
    resumed = np.random.default_rng(0)
    resumed.bit_generator.state = got_tr["rng"]
    assert np.array_equal(resumed.integers(0, 1 << 30, 64), rng.integers(0, 1 << 30, 64))


def test_checkpoint_version_is_checked():
    z = sg.pack_checkpoint({"step_count": np.array(0)}, {"step": 0})
    z["checkpoint_version"] = np.array(sg.CHECKPOINT_VERSION + 1)
    with pytest.raises(ValueError):
        sg.unpack_checkpoint(z)
