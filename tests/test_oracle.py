"""Pin the CPU oracle to the reference's own golden outputs and KAT."""
import numpy as np
import pytest

from conftest import dex_error
from uclchem_gb300.analysis import element_counts
from uclchem_gb300.params import ParameterError, make_params


def test_static_cloud_matches_golden(oracle, static_golden):
    """examples/example-output/static-full.dat rows <= 1e6 yr (config 1)."""
    phys, ab, flag, cnt = oracle.cloud({"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e6})
    g_phys, g_ab = static_golden["phys"], static_golden["abund"]
    assert flag == 0
    assert len(phys) == len(g_phys) == 47
    np.testing.assert_allclose(phys[:, 0], g_phys[:, 0], rtol=1e-4)
    np.testing.assert_allclose(phys[:, 1:7], g_phys[:, 1:7], rtol=5e-5)
    # the golden file prints 5 significant digits
    assert dex_error(ab, g_ab) < 1e-4
    sel = g_ab > 1e-25
    assert np.max(np.abs(ab[sel] - g_ab[sel]) / g_ab[sel]) < 1e-5


@pytest.mark.slow
def test_freefall_cloud_matches_golden(oracle, freefall_golden):
    """examples/example-output/phase1-full.dat: freefall 1e2 -> 1e5, densdot + Av updates."""
    phys, ab, flag, cnt = oracle.cloud({"initialDens": 1e2, "initialTemp": 10.0, "finalTime": 5e6,
                                        "freefall": True, "endAtFinalDensity": True, "finalDens": 1e5})
    g_phys, g_ab = freefall_golden["phys"], freefall_golden["abund"]
    assert flag == 0
    assert len(phys) == len(g_phys)
    np.testing.assert_allclose(phys[:, 1], g_phys[:, 1], rtol=1e-4)
    np.testing.assert_allclose(phys[:, 4], g_phys[:, 4], rtol=1e-4)
    assert dex_error(ab, g_ab) < 0.01


def test_ode_conservation_kat(oracle):
    """src/uclchem/tests.py:13-66: element-weighted ydot after a 1e3 yr freefall run."""
    pd = {"endatfinaldensity": False, "freefall": True, "initialdens": 1e4, "initialtemp": 10.0,
          "finaldens": 1e5, "finaltime": 1.0e3}
    phys, ab, flag, _ = oracle.cloud(pd)
    assert flag == 0
    ydot, flag2 = oracle.get_odes(pd, ab[-1])
    sp = oracle.tables.species
    for e in ["H", "N", "C", "O"]:
        assert abs(element_counts(sp, e) @ ydot[:len(sp)]) < 1e-15


def test_element_conservation_over_run(oracle):
    phys, ab, flag, _ = oracle.cloud({"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e6})
    sp = oracle.tables.species
    for e in ["H", "C", "N", "O", "S", "HE"]:
        tot = ab @ element_counts(sp, e)
        assert np.abs(tot / tot[0] - 1).max() < 1e-8


def test_parameter_parsing():
    p = make_params({"InitialDens": 1e5, "thermdesorb": False})
    assert p["initialDens"] == 1e5
    assert p["uvdesorb"] == 0 and p["thermdesorb"] == 1  # quirk Q2
    assert p["rout"] == float(np.float32(0.05))
    with pytest.raises(ParameterError):
        make_params({"nonsense": 1})
    with pytest.raises(ParameterError):
        make_params({"initialDens": 1, "initialdens": 2})


def test_failure_codes_from_host_injection(oracle):
    """Impossible step budget: DVODE returns ISTATE=-1, the retry loop shrinks
    targetTime and the model ends with INT_TOO_MANY_FAILS_ERROR (-5)."""
    import ctypes
    from uclchem_gb300.params import make_params as mp
    p = mp({"initialDens": 1e4, "finalTime": 1e3})
    p["mxstep"] = 1
    phys = np.zeros((64, 8))
    ab = np.zeros((64, oracle.nspec))
    nrows = ctypes.c_int(0)
    flag = oracle.lib.orc_cloud(oracle.net, p.ctypes.data, None, 64,
                                phys.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                ab.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(nrows), None)
    assert flag == -5
