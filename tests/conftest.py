import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fermi.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


_cache = {}


def inputs(n, seed=0, df=True):
    """Cached stand-in inputs: n = 1 README water, else seeded (H2O)n."""
    from fermicc.inputs import scf
    key = (n, seed, df)
    if key not in _cache:
        _cache[key] = scf.water_inputs(n, seed=seed, df=df)
    return _cache[key]


@pytest.fixture(scope="session")
def water_conv():
    return inputs(1, df=False)


@pytest.fixture(scope="session")
def water_df():
    return inputs(1, df=True)


@pytest.fixture(scope="session")
def dimer_df():
    return inputs(2, seed=0)
