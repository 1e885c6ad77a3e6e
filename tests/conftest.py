import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "geodesic-m_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C-ABI library)")
    config.addinivalue_line("markers", "slow: longer CPU-only check")


def fixture_path(name):
    return os.path.join(GOLDEN, f"{name}.npz")


@pytest.fixture
def load_fixture():
    from geodesic_cuda import amber

    def _load(name):
        atoms, topo, state, _ = amber.load_npz(fixture_path(name))
        return atoms, topo, state
    return _load
