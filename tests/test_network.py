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


def test_committed_tables_recompile_from_makerates_outputs():
    """The MakeRates hook is reproducible: compiling the reference's
    network.f90 + odes.f90 gives byte-identical device tables.  The UCLCHEM
    source tree is named by the UCLCHEM_REFERENCE_ROOT environment variable;
    the test is skipped where it is unset or lacks the MakeRates outputs."""
    import os
    import pytest
    from uclchem_gb300 import network
    root = os.environ.get("UCLCHEM_REFERENCE_ROOT")
    if not root:
        pytest.skip("UCLCHEM_REFERENCE_ROOT is not set")
    src = os.path.join(root, "src", "fortran_src")
    nf, of = os.path.join(src, "network.f90"), os.path.join(src, "odes.f90")
    if not (os.path.exists(nf) and os.path.exists(of)):
        pytest.skip("MakeRates outputs of the reference not present")
    blob = network.compile_network(nf, of).to_blob()
    with open(network.DEFAULT_BLOB, "rb") as f:
        assert f.read() == blob


def test_blob_records_are_well_formed(net):
    """UCLNET01: magic, then name[32] | kind u32 | count u64 | data records."""
    import struct
    from uclchem_gb300 import network
    data = open(network.DEFAULT_BLOB, "rb").read()
    assert data[:8] == b"UCLNET01"
    off, recs = 8, {}
    while off < len(data):
        name, kind, count = struct.unpack_from("<32sIQ", data, off)
        off += 44
        size = count * (4 if kind == 1 else 8)
        assert kind in (1, 2) and off + size <= len(data)
        recs[name.rstrip(b"\0").decode()] = (kind, count)
        off += size
    assert off == len(data)
    assert recs["dims"] == (1, 3) and recs["alpha"] == (2, net.nreac)
    assert recs["stoich_ptr"] == (1, net.nspec + 1) and recs["stoich_rx"][1] == len(net.stoich_rx)


def test_grid_parameters_are_seeded_and_in_range():
    from uclchem_gb300.params import grid_params
    a, b = grid_params(4096), grid_params(4096)
    assert a == b
    dens = np.array([d["initialDens"] for d in a])
    temp = np.array([d["initialTemp"] for d in a])
    zeta = np.array([d["zeta"] for d in a])
    rad = np.array([d["radfield"] for d in a])
    assert 1e2 <= dens.min() and dens.max() <= 1e7 and 10 <= temp.min() and temp.max() <= 50
    assert 1 <= zeta.min() and zeta.max() <= 1e3 and 1 <= rad.min() and rad.max() <= 1e3
    # log-uniform: about a fifth of the points per decade of density
    counts = np.histogram(np.log10(dens), bins=5, range=(2, 7))[0]
    assert (np.abs(counts / 4096 - 0.2) < 0.03).all()


def test_invariants_are_exactly_conserved_by_every_reaction(net):
    """The linear invariants the mixed path projects onto: element counts
    that every reaction conserves (integer check over the stoichiometry).
    H is not among them: a few freeze-outs hydrogenate (C2N -> #CH3CNH)."""
    from uclchem_gb300.analysis import element_counts
    inv = net.invariants()
    S = np.zeros((net.nspec, net.nreac), dtype=np.int64)
    for i in range(net.nspec):
        for e in range(net.stoich_ptr[i], net.stoich_ptr[i + 1]):
            S[i, net.stoich_rx[e]] += net.stoich_coef[e]
    assert inv.shape == (8, net.nspec)
    assert not (inv @ S).any()
    h = element_counts(net.species, "H")
    assert (h @ S).any()
    for el in ("HE", "C", "N", "O", "S", "SI", "MG", "CL"):
        assert any((row == element_counts(net.species, el)).all() for row in inv), el
