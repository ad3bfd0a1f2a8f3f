"""Kernel parity on the GPU: rate coefficients, RHS and analytic Jacobian
against the CPU oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import random_state
from uclchem_gb300.params import grid_params, make_param_array

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from uclchem_gb300 import _lib, network
    c = _lib.Context(network.DEFAULT_BLOB, device=0)
    yield c
    c.close()


def _states(net, oracle, n=6):
    """Elemental starts and evolved states for a few grid parameter sets."""
    dicts = grid_params(n, seed=11, final_time=1e4)
    dicts[0] = {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e4}
    ys = []
    for d in dicts:
        phys, ab, flag, _ = oracle.cloud(d, max_rows=64)
        y = np.zeros(net.neq)
        y[:net.nspec] = ab[len(ab) // 2]
        y[-1] = phys[len(ab) // 2, 1]
        ys.append(y)
    return dicts, np.array(ys)


def _av(oracle, d, y):
    """Av of the model at set-up (the oracle derives it from the parameters)."""
    return oracle.rates(d, y)[2][0]


def test_rates_match_oracle(ctx, oracle, net):
    dicts, ys = _states(net, oracle)
    params = make_param_array(dicts)
    av = np.array([_av(oracle, d, ys[k]) for k, d in enumerate(dicts)])
    phi = np.array([1e5, 3e3, 1e2, 1e6, 5e4, 1e5])[:len(dicts)]
    rates, ab, phi_out = ctx.rates(params, ys, av, phi)
    for k, d in enumerate(dicts):
        ref, ab_ref, phys = oracle.rates(dict(d), ys[k], phi=phi[k])
        np.testing.assert_array_equal(ref == 0.0, rates[k] == 0.0)
        nz = ref != 0.0
        rel = np.abs(rates[k][nz] - ref[nz]) / np.abs(ref[nz])
        assert rel.max() < 1e-12, (k, rel.max(), np.argmax(rel))
        np.testing.assert_allclose(ab[k], ab_ref, rtol=1e-15, atol=0)
        assert abs(phi_out[k] - phys[3]) <= 1e-13 * phys[3]


def test_rhs_matches_oracle(ctx, oracle, net):
    rng = np.random.default_rng(3)
    dicts, ys = _states(net, oracle)
    for extra in range(3):
        ys = np.vstack([ys, random_state(net, rng, n0=dicts[extra]["initialDens"])])
        dicts.append(dicts[extra])
    params = make_param_array(dicts)
    av = np.array([_av(oracle, d, ys[k]) for k, d in enumerate(dicts)])
    rates = 10.0 ** rng.uniform(-18, -8, (len(dicts), net.nreac))
    ydot = ctx.rhs(params, ys, rates, av)
    for k, d in enumerate(dicts):
        ref, scale = oracle.rhs(d, ys[k], rates[k])
        tol = 1e-12 * np.maximum(scale, np.abs(ref)) + 1e-300
        bad = np.abs(ydot[k] - ref) > tol
        assert not bad.any(), (k, np.nonzero(bad)[0][:10])


def test_jacobian_matches_finite_differences(ctx, oracle, net):
    dicts, ys = _states(net, oracle, n=3)
    params = make_param_array(dicts)
    av = np.array([_av(oracle, d, ys[k]) for k, d in enumerate(dicts)])
    rng = np.random.default_rng(5)
    rates = 10.0 ** rng.uniform(-16, -9, (len(dicts), net.nreac))
    J = ctx.jac(params, ys, rates, av)
    for k, d in enumerate(dicts):
        y = ys[k]
        n = net.neq
        Jfd = np.zeros((n, n))
        for j in range(n):
            # central differences are exact for the bilinear mass-action terms;
            # the floor keeps the step above the rounding of F for trace species
            h = 1e-5 * max(abs(y[j]), 1e-10)
            yp, ym = y.copy(), y.copy()
            yp[j] += h
            ym[j] -= h
            fp, _ = oracle.rhs(d, yp, rates[k])
            fm, _ = oracle.rhs(d, ym, rates[k])
            Jfd[:, j] = (fp - fm) / (yp[j] - ym[j])
        # compare in the error-weighted norm DVODE uses: rows by 1/ewt, columns by ewt
        w = 1.0 / (1e-8 * np.abs(y) + np.maximum(1e-14 * np.abs(y), 1e-25))
        Js = J[k] * w[:, None] / w[None, :]
        Jfs = Jfd * w[:, None] / w[None, :]
        err = np.abs(Js - Jfs)
        scale = np.abs(Jfs).max(axis=1, keepdims=True) + 1e-300
        assert (err / scale).max() < 1e-4, (k, np.unravel_index(np.argmax(err / scale), err.shape))
