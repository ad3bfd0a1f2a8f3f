"""Whole-model parity on the GPU: CLOUD models through ucl_solve_models (the
C ABI) against the oracle, the reference's golden output and conservation."""
import numpy as np
import pytest

from conftest import dex_error
from uclchem_gb300.analysis import element_counts
from uclchem_gb300.params import grid_params, make_param_array

pytestmark = pytest.mark.gpu

CONFIG1 = {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e6}
FREEFALL = {"initialDens": 1e2, "initialTemp": 10.0, "finalTime": 5e6, "freefall": True,
            "endAtFinalDensity": True, "finalDens": 1e5}


@pytest.fixture(scope="module")
def ctx():
    from uclchem_gb300 import _lib, network
    c = _lib.Context(network.DEFAULT_BLOB, device=0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def config1_oracle(oracle):
    return oracle.cloud(CONFIG1, max_rows=64)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_config1_matches_oracle_and_golden(ctx, oracle, config1_oracle, static_golden, precision):
    params = make_param_array([CONFIG1])
    phys, ab, nrows, flags, stats = ctx.solve_models(params, 64, precision=precision)
    ophys, oab, oflag, _ = config1_oracle
    n = int(nrows[0])
    assert flags[0] == 0 and n == len(ophys) == 47
    np.testing.assert_allclose(phys[0, :n, 0], ophys[:, 0], rtol=1e-12)
    np.testing.assert_allclose(phys[0, :n, 1:7], ophys[:, 1:7], rtol=1e-12)
    assert dex_error(ab[0, :n], oab) < 0.01
    assert dex_error(ab[0, :n], static_golden["abund"]) < 0.01


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_grid_points_match_oracle(ctx, oracle, precision):
    dicts = grid_params(6, seed=20261203, final_time=1e5)
    params = make_param_array(dicts)
    phys, ab, nrows, flags, stats = ctx.solve_models(params, 64, precision=precision)
    ophys, oab, onrows, oflags, _ = oracle.cloud_batch(dicts, max_rows=64)
    for k in range(len(dicts)):
        assert flags[k] == oflags[k] == 0
        assert nrows[k] == onrows[k]
        n = int(nrows[k])
        assert dex_error(ab[k, :n], oab[k, :n]) < 0.01, k


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_freefall_matches_golden(ctx, freefall_golden, precision):
    """examples/example-output/phase1-full.dat: freefall collapse 1e2 -> 1e5
    with densdot in the ODE system and the Av update between intervals."""
    phys, ab, nrows, flags, stats = ctx.solve_models(make_param_array([FREEFALL]), 256, precision=precision)
    g_phys, g_ab = freefall_golden["phys"], freefall_golden["abund"]
    n = int(nrows[0])
    assert flags[0] == 0 and n == len(g_phys)
    np.testing.assert_allclose(phys[0, :n, 1], g_phys[:, 1], rtol=1e-4)
    np.testing.assert_allclose(phys[0, :n, 4], g_phys[:, 4], rtol=1e-4)
    assert dex_error(ab[0, :n], g_ab) < 0.01


def test_element_conservation(ctx, net):
    """The network's conserved elements (every reaction conserves them) are
    conserved to 1e-10 relative at every row in both precisions; H, which a
    few hydrogenating freeze-outs create, to 1e-8 (the oracle's level)."""
    params = make_param_array([CONFIG1])
    inv = net.invariants()
    for precision in (0, 1):
        phys, ab, nrows, flags, stats = ctx.solve_models(params, 64, precision=precision)
        n = int(nrows[0])
        tot = ab[0, :n] @ inv.T
        assert np.abs(tot / tot[0] - 1).max() < 1e-10, precision
        h = ab[0, :n] @ element_counts(net.species, "H")
        assert np.abs(h / h[0] - 1).max() < 1e-8, precision


def test_failure_codes_from_host_injection(ctx):
    """MXSTEP=1 makes every DVODE call return ISTATE=-1; the retry loop then
    ends the model with INT_TOO_MANY_FAILS_ERROR, exactly as the oracle."""
    params = make_param_array([{"initialDens": 1e4, "finalTime": 1e3}])
    params[0]["mxstep"] = 1
    phys, ab, nrows, flags, stats = ctx.solve_models(params, 64, precision=1)
    assert flags[0] == -5
    params = make_param_array([CONFIG1])
    phys, ab, nrows, flags, stats = ctx.solve_models(params, 8, precision=1)
    assert flags[0] == -6 and nrows[0] == 8


def test_python_api_cloud_mirrors_reference_layout(oracle):
    """uclchem.model.cloud's calling convention (src/uclchem/model.py:227-316)
    on the device path: the [flag, abundances...] list, the array tuple, the
    parameter-error flag and a restart from a previous final abundance."""
    from uclchem_gb300 import model
    pd = {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e4}
    out = model.cloud(pd, out_species=["CO", "H2O"])
    assert out[0] == 0 and len(out) == 3 and min(out[1:]) > 0
    phys, chem, rates, start, flag = model.cloud(pd, return_array=True)
    assert flag == 0 and rates is None
    assert phys.shape[1:] == (1, 8) and chem.shape[1:] == (1, 335) and start.shape == (335,)
    ophys, oab, oflag, _ = oracle.cloud(pd, max_rows=64)
    assert dex_error(chem[:, 0, :], oab) < 0.01
    assert model.cloud({"notAParameter": 1.0})[0] == -1
    phys2, chem2, _, _, flag2 = model.cloud({"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e3},
                                             return_array=True, starting_chemistry=start)
    assert flag2 == 0 and np.allclose(chem2[0, 0, :], start, rtol=1e-6, atol=1e-20)


def test_empty_batches_and_invalid_arguments(ctx):
    """Edge cases at the C ABI: empty batches succeed without work; invalid
    precision, zero output rows and unsupported LU sizes are rejected with
    UCL_E_ARG before anything is launched."""
    from uclchem_gb300 import _lib
    phys, ab, nrows, flags, stats = ctx.solve_models(make_param_array([]), 8)
    assert phys.shape == (0, 8, 8) and ab.shape[0] == 0 and len(flags) == 0
    params = make_param_array([CONFIG1])
    with pytest.raises(_lib.UclError, match="-101"):
        ctx.solve_models(params, 8, precision=7)
    with pytest.raises(_lib.UclError, match="-101"):
        ctx.solve_models(params, 0)
    import torch
    m = torch.zeros((1, 338, 338), dtype=torch.float32, device="cuda")
    perm = torch.zeros((1, 338), dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.UclError, match="-101"):
        ctx.lu_factor_device(1, 338, _lib.PREC_MIXED, m.data_ptr(), perm.data_ptr(), info.data_ptr())
    ctx.lu_factor_device(0, 336, _lib.PREC_MIXED, m.data_ptr(), perm.data_ptr(), info.data_ptr())
