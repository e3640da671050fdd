import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def to_oracle_config(cfg):
    """RunConfig (product) -> oracle Config with the same fields."""
    from oracle import mattohf_oracle as O
    import dataclasses
    return O.Config(**{f.name: getattr(cfg, f.name) for f in dataclasses.fields(O.Config)})


@pytest.fixture(scope="session")
def built_lib():
    """Build (if needed) and load the CUDA library; fail loudly if that is impossible."""
    from mattohf_gb300 import build, _capi
    build.build()
    return _capi.load()
