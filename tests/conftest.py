import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def oracle_cpu():
    from oracle import build, cpu
    build.build_oracle()
    return cpu


@pytest.fixture(scope="session")
def ctx():
    """GPU context; the product has no CPU fallback, so a missing GPU is an error."""
    import focss_gb300 as fg
    c = fg.Context.default()
    return c


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


# SSMF of the benchmark configurations (SI units)
ALPHA = 0.2e-3 * np.log(10) / 10
BETA2 = -(1.55e-6 ** 2) * 17e-6 / (2 * 3.14159265358979323846264338 * 299792458.0)
GAMMA = 1.3e-3
F0 = 299792458.0 / 1.55e-6
