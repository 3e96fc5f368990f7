import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as _orc
    _orc.lib()
    return _orc


@pytest.fixture(scope="session")
def ctx():
    if not gpu_available():
        pytest.skip("no CUDA device")
    import vermeer_gb300 as vg
    c = vg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def host_ctx():
    import vermeer_gb300 as vg
    c = vg.Context(-1)
    yield c
    c.close()


def assert_hits_equal(got, ref, keys=("prim", "t", "u", "v", "w"), what=""):
    """Bit-exact comparison of hit streams (float compared by bit pattern)."""
    for k in keys:
        g = np.asarray(got[k])
        r = np.asarray(ref[k])
        if g.dtype == np.float32:
            g = g.view(np.uint32)
            r = r.view(np.uint32)
        bad = np.nonzero(g != r)[0]
        assert bad.size == 0, (f"{what} field {k}: {bad.size} of {g.size} rays differ; first {bad[:5]} "
                               f"got {np.asarray(got[k])[bad[:5]]} ref {np.asarray(ref[k])[bad[:5]]}")
