"""Seeded synthetic stiff mass-action networks that conserve elements and
charge: the uneven-size workload (N in {64, 128, 256, 512} species, about
10 N one- and two-body reactions) used to exercise the solver beyond the
default UCLCHEM network.

Species are small compositions of four elements (H, C, O, N) with charge 0
or +1, plus the electron.  Every reaction is checked to conserve each
element and the charge exactly (integer arithmetic):

  two-body  A + B -> C + D    flux = k2 * n * y_A * y_B   (k2 in cm^3 s^-1)
  one-body  A -> C + D        flux = k1 * y_A             (k1 in s^-1)

with y fractional abundances and n the density (cm^-3), the same flux forms
as UCLCHEM's two-body and cosmic-ray terms (odes.f90: RATE(j)*Y(a)*Y(b)*D and
RATE(j)*Y(a)).  Rate coefficients are log-uniform, k2 in 1e-20..1e-8 and k1
in 1e-17..1e-9; initial abundances log-uniform in 1e-12..1e-4 with H = 1.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

ELEMENTS = ("H", "C", "O", "N")
SIZES = (64, 128, 256, 512)


@dataclass
class SyntheticNetwork:
    names: List[str]
    comp: np.ndarray          # [N, 4] element counts
    charge: np.ndarray        # [N]
    reactants: np.ndarray     # [M, 2] (second = -1 for one-body)
    products: np.ndarray      # [M, 2]
    k: np.ndarray             # [M]
    density: float = 1.0e4
    # flux form and signed stoichiometric CSR (species-major)
    stoich_ptr: np.ndarray = field(default=None)
    stoich_rx: np.ndarray = field(default=None)
    stoich_coef: np.ndarray = field(default=None)

    @property
    def nspec(self) -> int:
        return len(self.names)

    @property
    def nreac(self) -> int:
        return len(self.k)

    def conserved(self) -> np.ndarray:
        """[5, N] element counts and charge per species."""
        return np.vstack([self.comp.T, self.charge[None, :]]).astype(np.int64)


def _name(c, q) -> str:
    s = "".join(f"{e}{'' if n == 1 else n}" for e, n in zip(ELEMENTS, c) if n > 0)
    return (s or "E") + ("+" if q > 0 else "-" if q < 0 else "")


def _species(n: int, rng: np.random.Generator):
    """n distinct compositions: the atoms, their ions and the electron first,
    the rest drawn from a lattice sized to n."""
    hmax, smax = (3, 8) if n <= 128 else (7, 8) if n <= 256 else (7, 11)
    lat = [(h, c, o, m) for h in range(hmax + 1) for c in range(4) for o in range(4) for m in range(3)
           if 0 < h + c + o + m <= smax]
    if 2 * len(lat) + 9 < n:
        raise ValueError(f"no {n} distinct compositions in the lattice")
    base = [((1, 0, 0, 0), 0), ((0, 1, 0, 0), 0), ((0, 0, 1, 0), 0), ((0, 0, 0, 1), 0),
            ((1, 0, 0, 0), 1), ((0, 1, 0, 0), 1), ((0, 0, 1, 0), 1), ((0, 0, 0, 1), 1), ((0, 0, 0, 0), -1)]
    chosen = set(base)
    order = rng.permutation(len(lat) * 2)
    for t in order:
        if len(chosen) >= n:
            break
        c = lat[t // 2]
        chosen.add((c, int(t % 2)))
    sp = base + sorted(chosen - set(base), key=lambda x: (sum(x[0]), x[0], x[1]))
    return sp[:n]


def make_network(n: int, seed: int = 20261203, density: float = 1.0e4) -> SyntheticNetwork:
    rng = np.random.default_rng(seed + n)
    sp = _species(n, rng)
    comp = np.array([c for c, _ in sp], dtype=np.int64)
    charge = np.array([q for _, q in sp], dtype=np.int64)
    index = {(tuple(c), int(q)): i for i, (c, q) in enumerate(zip(map(tuple, comp), charge))}
    target = 10 * n
    reacts, prods, ks = [], [], []
    seen = set()
    tries = 0
    while len(ks) < target and tries < 400 * target:
        tries += 1
        two = rng.uniform() < 0.7
        a = int(rng.integers(n))
        b = int(rng.integers(n)) if two else -1
        tot = comp[a] + (comp[b] if two else 0)
        q = charge[a] + (charge[b] if two else 0)
        # split the total into two existing species (C, D), C drawn at random
        cands = []
        for c in rng.permutation(n)[:64]:
            rest = tot - comp[c]
            if (rest < 0).any():
                continue
            key = (tuple(int(x) for x in rest), int(q - charge[c]))
            d = index.get(key)
            if d is not None and {int(c), d} != ({a, b} if two else {a}):
                cands.append((int(c), d))
        if not cands:
            continue
        c, d = cands[0]
        key = (min(a, b), max(a, b), min(c, d), max(c, d)) if two else (a, -1, min(c, d), max(c, d))
        if key in seen:
            continue
        seen.add(key)
        reacts.append((a, b))
        prods.append((c, d))
        ks.append(10 ** rng.uniform(-20, -8) if two else 10 ** rng.uniform(-17, -9))
    net = SyntheticNetwork(names=[_name(c, q) for c, q in zip(comp, charge)], comp=comp, charge=charge,
                           reactants=np.array(reacts, dtype=np.int64), products=np.array(prods, dtype=np.int64),
                           k=np.array(ks), density=density)
    _build_csr(net)
    return net


def _build_csr(net: SyntheticNetwork) -> None:
    rows: List[List[Tuple[int, int]]] = [[] for _ in range(net.nspec)]
    for r, ((a, b), (c, d)) in enumerate(zip(net.reactants, net.products)):
        for s in (a, b):
            if s >= 0:
                rows[s].append((r, -1))
        for s in (c, d):
            rows[s].append((r, +1))
    ptr = [0]
    rx, coef = [], []
    for lst in rows:
        for r, cf in lst:
            rx.append(r)
            coef.append(cf)
        ptr.append(len(rx))
    net.stoich_ptr = np.array(ptr, dtype=np.int64)
    net.stoich_rx = np.array(rx, dtype=np.int64)
    net.stoich_coef = np.array(coef, dtype=np.int64)


def initial_abundances(net: SyntheticNetwork, nsys: int, seed: int = 20261203) -> np.ndarray:
    rng = np.random.default_rng(seed + 7 * net.nspec)
    y = 10.0 ** rng.uniform(-12, -4, (nsys, net.nspec))
    y[:, 0] = 1.0  # H
    return y


def fluxes(net: SyntheticNetwork, y: np.ndarray) -> np.ndarray:
    a, b = net.reactants[:, 0], net.reactants[:, 1]
    f = net.k * y[..., a]
    two = b >= 0
    f = np.where(two, f * net.density * y[..., np.where(two, b, 0)], f)
    return f


def rhs(net: SyntheticNetwork, y: np.ndarray) -> np.ndarray:
    f = fluxes(net, y)
    out = np.zeros_like(y)
    for i in range(net.nspec):
        s0, s1 = net.stoich_ptr[i], net.stoich_ptr[i + 1]
        out[..., i] = (net.stoich_coef[s0:s1] * f[..., net.stoich_rx[s0:s1]]).sum(axis=-1)
    return out


def jacobian(net: SyntheticNetwork, y: np.ndarray) -> np.ndarray:
    """Dense dF/dy of one system (y: [N])."""
    n = net.nspec
    J = np.zeros((n, n))
    for r, ((a, b), (c, d)) in enumerate(zip(net.reactants, net.products)):
        if b >= 0:
            da = net.k[r] * net.density * y[b]
            db = net.k[r] * net.density * y[a]
        else:
            da, db = net.k[r], 0.0
        for s, sign in ((a, -1), (b, -1), (c, 1), (d, 1)):
            if s < 0:
                continue
            J[s, a] += sign * da
            if b >= 0:
                J[s, b] += sign * db
    return J


def to_network(net: SyntheticNetwork):
    """The synthetic network as a compiled :class:`uclchem_gb300.network.Network`
    (the table compiler's input form), so it loads through the same C ABI as
    a MakeRates network.  Every reaction sits in the two-body range with
    beta = gamma = 0, so its device rate is exactly alpha (the constant k);
    two-body fluxes have the RATE*D*Y*Y shape and one-body fluxes RATE*Y.
    There are no ices, no self-shielded photo reactions and no named species:
    the named-species slots point at the density slot, as UCLCHEM does for
    elements a network lacks, and the named reactions are absent (-1)."""
    from .network import (REACTION_PARAMS, SPECIES_PARAMS, RANGE_NAMES, Network)
    n, m = net.nspec, net.nreac
    empty_i = np.zeros(0, dtype=np.int32)
    empty_d = np.zeros(0, dtype=np.float64)
    ranges = {k: (99999, 99999) for k in RANGE_NAMES}
    ranges["twobodyReacs"] = (1, m)
    re = -np.ones((m, 3), dtype=np.int32)
    re[:, :2] = net.reactants
    pr = -np.ones((m, 4), dtype=np.int32)
    pr[:, :2] = net.products
    two = net.reactants[:, 1] >= 0
    shape = np.where(two, 0, 1).astype(np.int32)
    terms = []
    for r, ((a, b), (c, d)) in enumerate(zip(net.reactants, net.products)):
        for s, sign in ((a, -1), (b, -1), (c, 1), (d, 1)):
            if s >= 0:
                terms.append((s, sign, r, int(shape[r]), int(a), int(b)))
    out = Network(
        nspec=n, nreac=m, species=list(net.names),
        mass=np.ones(n), atom_counts=np.zeros(n, dtype=np.int32),
        surface_list=empty_i, bulk_list=empty_i, ice_list=empty_i, gas_ice_list=empty_i,
        refractory_list=empty_i, binding_energy=empty_d, formation_enthalpy=empty_d,
        three_phase=False, sp={k: n for k in SPECIES_PARAMS}, rx={k: -1 for k in REACTION_PARAMS},
        re=re, pr=pr, alpha=np.asarray(net.k, dtype=np.float64), beta=np.zeros(m), gama=np.zeros(m),
        min_temps=np.zeros(m), max_temps=np.full(m, 1e10), reduced_masses=np.zeros(m),
        extrapolate=np.ones(m, dtype=bool), freeze_partners=empty_i, gar_params=np.zeros((0, 7)),
        ranges=ranges, terms=np.array(terms, dtype=np.int32).reshape(-1, 6),
        swap_terms=np.zeros((0, 2), dtype=np.int32), tr_surface=empty_i, tr_bulk=empty_i,
    )
    out.flux_shape = shape
    out.flux_ya = np.ascontiguousarray(net.reactants[:, 0], dtype=np.int32)
    out.flux_yb = np.ascontiguousarray(net.reactants[:, 1], dtype=np.int32)
    out.stoich_ptr = np.ascontiguousarray(net.stoich_ptr, dtype=np.int32)
    out.stoich_rx = np.ascontiguousarray(net.stoich_rx, dtype=np.int32)
    out.stoich_coef = np.ascontiguousarray(net.stoich_coef, dtype=np.int32)
    out.invariant_counts = net.conserved()  # H, C, O, N counts and the charge
    return out


def write_blob(net: SyntheticNetwork, path: str) -> str:
    """Write the network's UCLNET01 blob (ucl_network_load's input)."""
    with open(path, "wb") as f:
        f.write(to_network(net).to_blob())
    return path


def start_vectors(net: SyntheticNetwork, nsys: int, seed: int = 20261203) -> np.ndarray:
    """[nsys, N+1] start vectors of the device solver: the seeded initial
    abundances and the network's density in the last (density) slot."""
    y = initial_abundances(net, nsys, seed)
    return np.concatenate([y, np.full((nsys, 1), net.density)], axis=1)
