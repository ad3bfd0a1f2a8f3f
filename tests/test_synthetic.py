"""Synthetic mass-action networks (uneven sizes N = 64..512, ~10 N
reactions): generator invariants, the host RHS/Jacobian, and the oracle's
DVODE on them, cross-checked against independent stiff integrators (ODEPACK's
LSODA and scipy's BDF)."""
import numpy as np
import pytest

from uclchem_gb300 import synthetic as S


@pytest.mark.parametrize("n", S.SIZES)
def test_every_reaction_conserves_elements_and_charge(n):
    net = S.make_network(n)
    assert net.nspec == n and net.nreac == 10 * n
    E = net.conserved()
    lhs = E[:, net.reactants[:, 0]] + np.where(net.reactants[:, 1] >= 0, E[:, net.reactants[:, 1]], 0)
    rhs = E[:, net.products[:, 0]] + E[:, net.products[:, 1]]
    np.testing.assert_array_equal(lhs, rhs)
    assert (net.k > 0).all()
    two = net.reactants[:, 1] >= 0
    assert 1e-20 <= net.k[two].min() and net.k[two].max() <= 1e-8
    assert 1e-17 <= net.k[~two].min() and net.k[~two].max() <= 1e-9


def test_rhs_conserves_and_jacobian_matches_differences(oracle_ma64):
    net, orc = oracle_ma64
    y = S.initial_abundances(net, 3)
    f = S.rhs(net, y)
    E = net.conserved().astype(float)
    assert np.abs(f @ E.T).max() <= 1e-13 * np.abs(f).max()
    np.testing.assert_allclose(orc.rhs(y[0]), f[0], rtol=1e-12, atol=1e-300)
    J = S.jacobian(net, y[0])
    # independent assembly through the species-major CSR: J_ij = sum_e coef_e d flux_rx(e) / d y_j
    n, yy = net.nspec, y[0]
    Jc = np.zeros((n, n))
    for i in range(n):
        for e in range(net.stoich_ptr[i], net.stoich_ptr[i + 1]):
            r, cf = net.stoich_rx[e], net.stoich_coef[e]
            a, b = net.reactants[r]
            if b >= 0:
                Jc[i, a] += cf * net.k[r] * net.density * yy[b]
                Jc[i, b] += cf * net.k[r] * net.density * yy[a]
            else:
                Jc[i, a] += cf * net.k[r]
    np.testing.assert_allclose(J, Jc, rtol=1e-12, atol=1e-12 * np.abs(Jc).max())
    # and a directional central difference (exact up to rounding for this quadratic F)
    v = yy / np.linalg.norm(yy)
    h = 1e-6 * np.linalg.norm(yy)
    fd = (S.rhs(net, yy + h * v) - S.rhs(net, yy - h * v)) / (2 * h)
    assert np.linalg.norm(J @ v - fd) <= 1e-6 * np.linalg.norm(fd)


@pytest.fixture(scope="module")
def oracle_ma64():
    from oracle.oracle import MassActionOracle
    net = S.make_network(64)
    return net, MassActionOracle(net)


def test_oracle_dvode_conserves_and_agrees_with_independent_integrators(oracle_ma64):
    scipy_integrate = pytest.importorskip("scipy.integrate")
    net, orc = oracle_ma64
    y0 = S.initial_abundances(net, 1)[0]
    tout = 3.16e7 * np.array([1e2, 1e3, 1e4])
    yo, rc, cnt = orc.solve(y0, tout)
    assert rc == 0 and cnt[0] > 0
    E = net.conserved().astype(float)
    tot0 = E @ y0
    for row in yo:
        tot = E @ row
        sel = np.abs(tot0) > 1e-12
        assert np.abs(tot[sel] / tot0[sel] - 1).max() < 1e-6
    # independent stiff integrators (ODEPACK's LSODA, scipy's own BDF) with
    # the analytic Jacobian and the same tolerances
    atol = np.maximum(1e-14 * y0, 1e-25)
    for method in ("LSODA", "BDF"):
        r = scipy_integrate.solve_ivp(lambda t, y: S.rhs(net, y), (0.0, tout[-1]), y0, method=method, rtol=1e-8,
                                      atol=atol, jac=lambda t, y: S.jacobian(net, y), t_eval=tout)
        assert r.success, r.message
        ys = r.y[:, -1]
        sel = (ys > 1e-14) | (yo[-1] > 1e-14)
        dex = np.abs(np.log10(np.maximum(ys[sel], 1e-300)) - np.log10(np.maximum(yo[-1][sel], 1e-300)))
        assert dex.max() < 1e-4, (method, dex.max())


def test_oracle_reports_dvode_failure_codes(oracle_ma64):
    """MXSTEP = 1 makes DVODE stop with ISTATE = -1 (too much work), which the
    mass-action driver returns unchanged."""
    net, orc = oracle_ma64
    y0 = S.initial_abundances(net, 1)[0]
    yo, rc, cnt = orc.solve(y0, [3.16e7 * 1e4], mxstep=1)
    assert rc == -1


@pytest.mark.parametrize("n", S.SIZES)
def test_synthetic_blob_loads_through_the_c_abi(n, tmp_path):
    """The table compiler's form of a synthetic network (to_network) is a
    valid UCLNET01 blob: the library's host loader reads it with the right
    sizes, every reaction is a constant-rate two-body-range entry and the
    flux shapes are RATE*D*Y*Y / RATE*Y."""
    import ctypes
    from uclchem_gb300 import _lib
    net = S.make_network(n)
    comp = S.to_network(net)
    two = net.reactants[:, 1] >= 0
    np.testing.assert_array_equal(comp.flux_shape, np.where(two, 0, 1))
    assert comp.ranges["twobodyReacs"] == (1, net.nreac)
    assert (comp.beta == 0).all() and (comp.gama == 0).all() and comp.extrapolate.all()
    assert set(comp.sp.values()) == {n} and set(comp.rx.values()) == {-1}
    path = S.write_blob(net, str(tmp_path / f"syn{n}.uclnet"))
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ucl_network_load(path.encode(), ctypes.byref(h)) == 0
    try:
        assert lib.ucl_network_nspec(h) == n and lib.ucl_network_nreac(h) == net.nreac
    finally:
        lib.ucl_network_free(h)


def test_oracle_cloud_schedule_on_a_synthetic_network(oracle_ma64):
    """orc_ma_cloud (the check for the GPU's generic-network path): the
    CLOUD output times to 1e6 yr, success, and element/charge totals
    conserved to 1e-10 of their largest absolute entry."""
    net, orc = oracle_ma64
    y0 = S.start_vectors(net, 1)[0]
    assert y0[-1] == net.density and y0.shape == (net.nspec + 1,)
    tyr, yout, flag, cnt = orc.cloud(y0, final_time_yr=1e6, max_rows=64)
    assert flag == 0 and len(tyr) == 47 and tyr[-1] == 1e6 and cnt[0] > 0
    tot = yout @ net.conserved().astype(float).T
    scale = np.abs(yout[0][None, :] * np.abs(net.conserved()).astype(float)).sum(axis=1)
    assert (np.abs(tot - tot[0]) / scale).max() < 1e-10
