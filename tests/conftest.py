import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The reference tree, present only where the fixtures are made; its location
# is the oracle build recipe's (GI_REFERENCE_ROOT overrides it).  Tests that
# read it skip elsewhere.
from oracle.build_oracle import REFERENCE_ROOT as REFERENCE  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    # Build (incrementally) the library and the oracle before any test imports them.
    from globalillumination_gb300.build import build_library
    from oracle.build_oracle import build_oracle, build_scene_ref

    build_library()
    build_oracle()
    build_scene_ref()  # the reference's own scene C++, where its tree is present


def has_reference() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "Configs"))


@pytest.fixture(scope="session")
def cuda_ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import globalillumination_gb300 as gi

    ctx = gi.Context(0)
    yield ctx
    ctx.close()
