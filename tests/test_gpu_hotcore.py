"""The hot-core physics module on the device (hotcore.f90: the temperature
ramp of a protostar and its output schedule) against the oracle's runs of
the same models (tests/golden/hotcore_models.npz, made by
tests/golden/make_hotcore.py), both precisions, through the C ABI: the
oracle's flag, a common row at every output time up to the first MXSTEP
stop of either run, at common rows the gas temperature and every species
above 1e-14 within 0.01 dex, the network's invariants conserved;
and the Python ``hot_core`` calling convention."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, dex_error
from uclchem_gb300.params import make_param_array

pytestmark = pytest.mark.gpu

FIX = os.path.join(GOLDEN, "hotcore_models.npz")
ROWS = 600
PARAMS = {"initialDens": 1e5, "initialTemp": 10.0, "finalTime": 5e4}


def _next_time(ty):
    """The hot-core module's next output time (yr), hotcore.f90:50-66."""
    for lim, step in ((1.0e6, 1.0e5), (1.0e5, 1.0e4), (1.0e4, 1000.0), (1000, 100.0), (100, 10.0)):
        if ty > lim:
            return ty + step
    return ty * 10.0 if ty > 0.0 else 1.0e-7


def _regular_prefix(t):
    n = 1
    while n < len(t) and abs(t[n] - _next_time(t[n - 1])) <= 1e-9 * t[n]:
        n += 1
    return n


def _common_rows(t_a, t_b):
    ia, ib = [], []
    j = 0
    for i, t in enumerate(t_a):
        while j < len(t_b) and t_b[j] < t * (1 - 1e-12):
            j += 1
        if j < len(t_b) and abs(t_b[j] - t) <= 1e-12 * max(t, 1.0):
            ia.append(i)
            ib.append(j)
    return np.array(ia, dtype=int), np.array(ib, dtype=int)


@pytest.fixture(scope="module")
def fx():
    if not os.path.exists(FIX):
        pytest.fail(f"fixture missing: {FIX}")
    return np.load(FIX)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_hot_core_matches_oracle(fx, net, precision):
    from uclchem_gb300 import _lib, network
    # the plain-FP64 path runs the first model only (the 25 Msun ramp takes
    # ~3e5 steps; its mixed run is compared)
    m = len(fx["temp_indx"]) if precision == 1 else 1
    params = make_param_array([PARAMS] * m)
    params["hotcore"] = fx["temp_indx"][:m]
    params["maxTemperature"] = fx["max_temperature"][:m]
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    try:
        ph, ab, nr, fl, st = ctx.solve_models(params, ROWS, precision=precision)
    finally:
        ctx.close()
    inv = net.invariants().T
    for k in range(m):
        r, n = int(fx["nrows"][k]), int(nr[k])
        assert fl[k] == fx["flag"][k] == 0, (k, fl[k])
        gt, ot = ph[k, :n, 0], fx["tyears"][k, :r]
        gi, oi = _common_rows(gt, ot)
        # every row up to the first MXSTEP stop of either run (a stop ends
        # its interval early and the schedule runs on from there)
        assert len(gi) >= min(_regular_prefix(gt), _regular_prefix(ot)), (k, len(gi), n, r)
        np.testing.assert_allclose(ph[k, gi, 2], fx["gas_temp"][k, oi], rtol=1e-12)
        np.testing.assert_array_equal(ph[k, :n, 3], ph[k, :n, 2])  # dustTemp = gasTemp
        oab = 10.0 ** (fx["log10_mdex"][k, oi].astype(np.float64) / 1000.0)
        d = dex_error(ab[k, gi], oab)
        assert d < 0.01, (k, d)
        tot = ab[k, :n] @ inv
        assert np.abs(tot / tot[0] - 1).max() < 1e-10, k


def test_python_hot_core_call(fx):
    """uclchem.model.hot_core(temp_indx, max_temperature, ...) with the
    reference's argument order and outputs; a temp_indx beyond the six
    masses fails at start-up (PHYSICS_INIT_ERROR)."""
    from uclchem_gb300 import model
    phys, chem, rates, start, flag = model.hot_core(int(fx["temp_indx"][0]), float(fx["max_temperature"][0]),
                                                    PARAMS, return_array=True, timepoints=ROWS - 1)
    gi, oi = _common_rows(phys[:, 0, 0], fx["tyears"][0, : int(fx["nrows"][0])])
    assert flag == 0 and phys.shape[1:] == (1, 8) and len(gi) > 40
    np.testing.assert_allclose(phys[gi, 0, 2], fx["gas_temp"][0, oi], rtol=1e-12)
    assert model.hot_core(7, 300.0, PARAMS) == [-2]
