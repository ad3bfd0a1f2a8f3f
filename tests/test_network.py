"""Network table compiler: structure and the flux regrouping of GETYDOT."""
import numpy as np

from conftest import random_state


def test_default_network_shape(net):
    assert net.nspec == 335 and net.neq == 336 and net.nreac == 3203
    assert len(net.terms) == 11061
    assert len(net.swap_terms) == 83
    assert net.species[net.sp["nelec"]] == "E-"
    assert net.species[net.sp["nsurface"]] == "SURFACE"
    assert net.ranges["twobodyReacs"] == (1236, 3203)
    assert (net.flux_shape >= 0).all()
    # stoichiometric rows: merged duplicates only
    assert len(net.stoich_rx) == 10929


def _flux_rhs(net, y, rate):
    """ydot from per-reaction fluxes and the signed stoichiometry CSR."""
    D = y[-1]
    sm = max(1e-30, y[net.sp["nsurface"]])
    sb = max(1e-30, y[net.sp["nbulk"]])
    PI = float(np.float32(3.141592654))
    GDR = (4.0 * PI * (1e-5 * 1e-5 * 1e-5) * 3.0 * 100.0) / (3.0 * 1.66053892e-24)
    NSPG = 1e-5 * 1e-5 * 1.5e15 * 4.0 * PI
    blr = min(1.0, NSPG / (GDR * sb))
    sh, a, b = net.flux_shape, net.flux_ya, net.flux_yb
    ya = y[a]
    yb = np.where(b >= 0, y[np.maximum(b, 0)], 1.0)
    dpow = np.array([1, 0, 1, 0, 0, 0, 0, 1, 0, 1])[sh]
    f = rate * ya * np.where(np.isin(sh, [0, 4, 5, 7, 9]), yb, 1.0) * np.where(dpow == 1, D, 1.0)
    f = np.where(np.isin(sh, [5, 6]), f * blr, f)
    swap = f[net.swap_terms[:, 0]].sum()
    f = np.where(sh == 8, f * swap, f)
    f = np.where(np.isin(sh, [3, 7, 8, 9]), f / sm, f)
    ydot = np.zeros(net.neq)
    for i in range(net.nspec):
        s, e = net.stoich_ptr[i], net.stoich_ptr[i + 1]
        ydot[i] = (net.stoich_coef[s:e] * f[net.stoich_rx[s:e]]).sum()
    ns, nb = net.sp["nsurface"], net.sp["nbulk"]
    y335 = ydot[net.surface_list].sum()
    if y335 < 0:
        sc = min(1.0, sb / sm)
        t = y335 * sc * y[net.bulk_list] / sb
    else:
        sc = 0.5 * GDR / NSPG
        t = y335 * sc * y[net.surface_list]
    ydot[net.surface_list] -= t
    ydot[net.bulk_list] += t
    ydot[nb] = ydot[net.bulk_list].sum()
    ydot[ns] = ydot[net.surface_list].sum()
    return ydot


def test_flux_form_reproduces_term_for_term_rhs(net, oracle):
    """Per-reaction fluxes + signed CSR == odes.f90 term for term (to rounding)."""
    rng = np.random.default_rng(7)
    for trial in range(6):
        y = random_state(net, rng)
        pd = {"initialDens": y[-1]}
        rates = 10.0 ** rng.uniform(-20, -8, net.nreac)
        h2, co = oracle.photo_rates(pd, y)
        rates[net.rx["nR_H2_hv"]] = h2
        rates[net.rx["nR_CO_hv"]] = co
        ydot_ref, scale = oracle.rhs(pd, y, rates)
        ydot_flux = _flux_rhs(net, y, rates)
        tol = 1e-12 * np.maximum(scale, np.abs(ydot_ref)) + 1e-300
        assert np.all(np.abs(ydot_flux - ydot_ref)[:net.nspec] <= tol[:net.nspec])
