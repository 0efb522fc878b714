import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    O.lib()
    return O


@pytest.fixture(scope="session")
def built_lib():
    from omg_audio_gb300 import build
    build.build()
    from omg_audio_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def ctx(built_lib):
    """A context with the reference's default constants (300 x 10 ms bins)."""
    from omg_audio_gb300 import Context, TraceConfig
    c = Context(TraceConfig())
    yield c
    c.close()


@pytest.fixture(scope="session")
def ctx_c1(built_lib):
    """Config-1 constants: 2000 x 1 ms bins, 2 s, 200 bounces, floor 1e-6."""
    from omg_audio_gb300 import Context, TraceConfig
    c = Context(TraceConfig(n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200, energy_floor=1e-6))
    yield c
    c.close()


@pytest.fixture(scope="session")
def ctx_tie(built_lib):
    """Config-1 constants with the precision-independent near-tie rule."""
    from omg_audio_gb300 import Context, TraceConfig
    c = Context(TraceConfig(n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200, energy_floor=1e-6,
                            tie_mode=1))
    yield c
    c.close()
