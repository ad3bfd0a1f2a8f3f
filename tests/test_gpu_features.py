"""Reference options on the device path, each against the oracle through the
C ABI: the rates array (returnRates, io.f90:89-93), enforceChargeConservation
(chemistry.f90:287-291, 333-335), improvedH2CRPDissociation with
cosmicRayAttenuation (rates.f90:38-41, physics-core.f90:121-157) and the
start-up rejections of coreInitializePhysics (physics-core.f90:55-64)."""
import numpy as np
import pytest

from conftest import dex_error
from uclchem_gb300.params import make_param_array

pytestmark = pytest.mark.gpu

SHORT = {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e5}


@pytest.fixture(scope="module")
def ctx():
    from uclchem_gb300 import _lib, network
    c = _lib.Context(network.DEFAULT_BLOB, device=0)
    yield c
    c.close()


def _rate_dex(a, b, floor=1e-30):
    """max |log10 a - log10 b| where both exceed floor, and the count of
    entries where exactly one of them is zero."""
    both = (a > floor) & (b > floor)
    d = np.abs(np.log10(a[both]) - np.log10(b[both]))
    return (float(d.max()) if d.size else 0.0), int(((a > floor) != (b > floor)).sum())


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_rates_rows_match_oracle(ctx, oracle, precision):
    """Row r of the rates array is rate() at output time: zero at row 0, then
    the interval's calculateReactionRates values with the H2 and CO
    photodissociation rates of the last F evaluation."""
    params = make_param_array([SHORT])
    phys, ab, nrows, flags, stats, rates = ctx.solve_models(params, 64, precision=precision, rates=True)
    ophys, oab, oflag, _, orates = oracle.cloud(SHORT, max_rows=64, rates=True)
    n = int(nrows[0])
    assert flags[0] == 0 and oflag == 0 and n == len(orates)
    assert not rates[0, 0].any() and not orates[0].any()
    assert not rates[0, n:].any()
    d, flips = _rate_dex(rates[0, 1:n], orates[1:n])
    assert d < 0.01 and flips == 0, (d, flips)
    assert dex_error(ab[0, :n], oab) < 0.01


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_charge_conservation_is_enforced(ctx, oracle, net, precision):
    """With enforceChargeConservation the electron abundance equals the sum
    of the positive ions after every interval (to 1e-10 relative), and the
    abundances match the oracle's run with the same option."""
    params = make_param_array([SHORT])
    params[0]["enforceChargeConservation"] = 1
    phys, ab, nrows, flags, stats = ctx.solve_models(params, 64, precision=precision)
    ophys, oab, oflag, _ = oracle.cloud(params[0], max_rows=64)
    n = int(nrows[0])
    assert flags[0] == 0 and oflag == 0 and n == len(oab)
    ions = [i for i, s in enumerate(net.species) if "+" in s]
    e = net.species.index("E-")
    rows = ab[0, 1:n]
    charge = rows[:, ions].sum(axis=1)
    assert (np.abs(rows[:, e] - charge) / charge).max() < 1e-10
    assert dex_error(ab[0, :n], oab) < 0.01


def test_improved_h2_crp_dissociation(ctx, oracle, net):
    """improvedH2CRPDissociation with cosmicRayAttenuation: the H2 CR
    dissociation rate is h2CRPRate, zero in the first interval (no physics
    update yet) and then the column-density fit of ionizationDependency."""
    from oracle.oracle import Oracle  # noqa: F401  (the fixture is the oracle)
    pd = dict(SHORT, cosmicRayAttenuation=True, improvedH2CRPDissociation=True, ionModel="H")
    params = make_param_array([pd])
    phys, ab, nrows, flags, stats, rates = ctx.solve_models(params, 64, precision=1, rates=True)
    ophys, oab, oflag, _, orates = oracle.cloud(pd, max_rows=64, rates=True)
    n = int(nrows[0])
    assert flags[0] == 0 and oflag == 0 and n == len(oab)
    j = net.rx["nR_H2_crp"]
    assert rates[0, 1, j] == 0.0 and orates[1, j] == 0.0
    assert rates[0, 2, j] > 0.0
    np.testing.assert_allclose(rates[0, 2:n, j], orates[2:n, j], rtol=1e-6)
    assert dex_error(ab[0, :n], oab) < 0.01


@pytest.mark.parametrize("opts", [{"improvedH2CRPDissociation": True},
                                  {"ionModel": "X"},
                                  {"points": 2}], ids=["h2crp-without-attenuation", "bad-ion-model", "points"])
def test_startup_rejections(ctx, oracle, opts):
    """coreInitializePhysics's checks give PHYSICS_INIT_ERROR (-2) and no
    rows, in the device path and in the oracle alike."""
    pd = dict(SHORT, **opts)
    phys, ab, nrows, flags, stats = ctx.solve_models(make_param_array([pd]), 8, precision=1)
    assert flags[0] == -2 and nrows[0] == 0
    assert oracle.cloud(pd, max_rows=8)[2] == -2


def test_python_cloud_returns_rates(oracle):
    """uclchem.model.cloud(..., return_array=True, return_rates=True) returns
    the rates array [rows, points, nreac] as the reference does."""
    from uclchem_gb300 import model
    phys, chem, rates, start, flag = model.cloud(SHORT, return_array=True, return_rates=True)
    assert flag == 0 and rates.shape == (phys.shape[0], 1, 3203)
    assert not rates[0].any() and rates[1:].any()
    with pytest.raises(AssertionError):
        model.cloud(SHORT, return_rates=True)
