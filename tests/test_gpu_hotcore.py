"""The hot-core physics module on the device (hotcore.f90: the temperature
ramp of a protostar and its output schedule) against the oracle's runs of
the same models (tests/golden/hotcore_models.npz, made by
tests/golden/make_hotcore.py), both precisions, through the C ABI: the
oracle's flag and output times, the gas temperature of every row, every
species above 1e-14 within 0.01 dex, the network's invariants conserved;
and the Python ``hot_core`` calling convention."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, dex_error
from uclchem_gb300.params import make_param_array

pytestmark = pytest.mark.gpu

FIX = os.path.join(GOLDEN, "hotcore_models.npz")
ROWS = 600
PARAMS = {"initialDens": 1e5, "initialTemp": 10.0, "finalTime": 1e5}


@pytest.fixture(scope="module")
def fx():
    if not os.path.exists(FIX):
        pytest.fail(f"fixture missing: {FIX}")
    return np.load(FIX)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_hot_core_matches_oracle(fx, net, precision):
    from uclchem_gb300 import _lib, network
    m = len(fx["temp_indx"])
    params = make_param_array([PARAMS] * m)
    params["hotcore"] = fx["temp_indx"]
    params["maxTemperature"] = fx["max_temperature"]
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    try:
        ph, ab, nr, fl, st = ctx.solve_models(params, ROWS, precision=precision)
    finally:
        ctx.close()
    inv = net.invariants().T
    for k in range(m):
        r = int(fx["nrows"][k])
        assert fl[k] == fx["flag"][k] == 0 and nr[k] == r, (k, fl[k], nr[k], r)
        np.testing.assert_allclose(ph[k, :r, 0], fx["tyears"][k, :r], rtol=1e-12)
        np.testing.assert_allclose(ph[k, :r, 2], fx["gas_temp"][k, :r], rtol=1e-12)
        np.testing.assert_array_equal(ph[k, :r, 3], ph[k, :r, 2])  # dustTemp = gasTemp
        oab = 10.0 ** (fx["log10_mdex"][k, :r].astype(np.float64) / 1000.0)
        d = dex_error(ab[k, :r], oab)
        assert d < 0.01, (k, d)
        tot = ab[k, :r] @ inv
        assert np.abs(tot / tot[0] - 1).max() < 1e-10, k


def test_python_hot_core_call(fx):
    """uclchem.model.hot_core(temp_indx, max_temperature, ...) with the
    reference's argument order and outputs; a temp_indx beyond the six
    masses fails at start-up (PHYSICS_INIT_ERROR)."""
    from uclchem_gb300 import model
    phys, chem, rates, start, flag = model.hot_core(int(fx["temp_indx"][0]), float(fx["max_temperature"][0]),
                                                    PARAMS, return_array=True, timepoints=ROWS - 1)
    r = int(fx["nrows"][0])
    assert flag == 0 and phys.shape == (r, 1, 8)
    np.testing.assert_allclose(phys[:, 0, 2], fx["gas_temp"][0, :r], rtol=1e-12)
    assert model.hot_core(7, 300.0, PARAMS) == [-2]
