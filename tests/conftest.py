import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O
    return O


@pytest.fixture(scope="session")
def engine_lib():
    from seisfat2d_gb300 import build as eb
    eb.build()
    from seisfat2d_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def exes(engine_lib):
    """The C++ drivers (seisfat2d_gb300/host), built against the engine library."""
    from seisfat2d_gb300.host import build as hb
    out = hb.build()
    return {k: os.path.join(out, k) for k in ("modeling.exe", "inversion.exe", "traveltime_tables.exe",
                                              "migration.exe")}
