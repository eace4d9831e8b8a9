import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path)")


def has_reference_sources() -> bool:
    from oracle import oracle
    return os.path.isdir(oracle.REFERENCE_SOURCES)


@pytest.fixture(scope="session")
def oracle_lib():
    """Builds the C restatement (and the reference library where its sources exist)."""
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def native_lib():
    from hamstr_oop_gb300 import native
    return native.load(build_if_missing=True)


@pytest.fixture
def make_case(tmp_path):
    """make_case(ni, nj, **inputs) -> case directory in a fresh temp dir."""
    from hamstr_oop_gb300 import meshgen
    counter = [0]

    def _make(ni, nj, **inputs):
        counter[0] += 1
        d = tmp_path / ("case%d_%dx%d" % (counter[0], ni, nj))
        return meshgen.make_case(str(d), ni, nj, **inputs)
    return _make
