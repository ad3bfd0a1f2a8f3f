import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than ~20 s on the CPU")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def net():
    from uclchem_gb300.network import load_default
    return load_default()


@pytest.fixture(scope="session")
def static_golden():
    return np.load(os.path.join(GOLDEN, "static_cloud.npz"))


@pytest.fixture(scope="session")
def freefall_golden():
    return np.load(os.path.join(GOLDEN, "freefall_cloud.npz"))


def dex_error(a, b, floor=1e-14):
    """max |log10 a - log10 b| over entries where either side exceeds floor."""
    a = np.asarray(a)
    b = np.asarray(b)
    sel = (a > floor) | (b > floor)
    if not sel.any():
        return 0.0
    d = np.abs(np.log10(np.maximum(a, 1e-300)) - np.log10(np.maximum(b, 1e-300)))
    return float(np.where(sel, d, 0.0).max())


def random_state(net, rng, n0=None):
    """A plausible abundance vector: log-uniform 1e-20..1e-4, H/H2 large, with
    surface/bulk totals consistent with the species."""
    y = 10.0 ** rng.uniform(-20, -4, net.neq)
    y[net.sp["nh"]] = rng.uniform(0.01, 0.5)
    y[net.sp["nh2"]] = rng.uniform(0.2, 0.5)
    y[net.sp["nhe"]] = 0.1
    y[net.sp["nsurface"]] = y[net.surface_list].sum()
    y[net.sp["nbulk"]] = y[net.bulk_list].sum()
    y[net.neq - 1] = n0 if n0 is not None else 10.0 ** rng.uniform(2, 7)
    return y
