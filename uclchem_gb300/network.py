"""MakeRates network -> device table compiler.

The reference compiles its chemical network at MakeRates time into two Fortran
files: ``network.f90`` (PARAMETER arrays: species, reactant/product indices,
Arrhenius coefficients, reaction-type index ranges; written by
``src/uclchem/makerates/io_functions.py:801-951``) and ``odes.f90`` (the
generated ``GETYDOT`` right-hand side, ``io_functions.py:533-661`` /
``reaction.py:779-819``).  This module reads those two files as they are and
produces a :class:`Network` holding

* the reaction tables that ``calculateReactionRates`` (``rates.f90:21-343``)
  consumes, in 0-based form;
* the generated RHS as an ordered term list (species row, LOSS/PROD, rate
  index, term shape, reactant slots) so a CPU evaluator can reproduce
  ``GETYDOT`` term for term (``odes.f90:6-5181``);
* the flux form the GPU uses: one flux per reaction (the product of its rate,
  density power, reactant abundances and ice modifiers) and a species-row CSR
  of signed stoichiometric coefficients, checked here to be an exact
  regrouping of the generated terms;
* the surface/bulk transfer branch (``odes.f90:4815-5180``).

``network.f90`` is the source of truth for coefficients: it stores them at 5
significant digits (``io_functions.py:1021``), which is what the compiled
reference integrates with.

The compiled tables are stored as a plain ``.npz`` (for Python) and as a flat
binary blob (``UCLNET01``) that the C ABI loader reads, so a Fortran host can
load a network without Python.
"""
from __future__ import annotations

import os
import re
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Tuple

import numpy as np

# Reaction-type index ranges in the order network.f90 declares them
# (network.f90:5147-5169).  Values are Fortran 1-based inclusive pairs;
# 99999 marks an absent type.
RANGE_NAMES = [
    "photonReacs", "crpReacs", "crphotReacs", "freezeReacs", "desorbReacs",
    "thermReacs", "desoh2Reacs", "descrReacs", "deuvcrReacs", "h2formReacs",
    "erReacs", "erdesReacs", "lhReacs", "lhdesReacs", "bulkswapReacs",
    "surfswapReacs", "ionopol1Reacs", "ionopol2Reacs", "crsReacs",
    "exsolidReacs", "exrelaxReacs", "garReacs", "twobodyReacs",
]

# Named species indices used by the chemistry (network.f90:4-8).  Elements
# absent from the network point at NEQ (the density slot, quirk of the
# reference: they are written at initialisation and then overwritten).
SPECIES_PARAMS = [
    "ncx", "nhx", "nh2", "nhe", "nhex", "nn", "nnx", "no", "nox", "nc", "nsix",
    "nsx", "nh2o", "nch3oh", "ncl", "nclx", "nco", "nmg", "nmgx", "ngh", "ngh2",
    "ngn", "ngo", "ngoh", "nsurface", "nbulk", "nh", "nd", "nf", "np", "ns",
    "nli", "nna", "nsi", "npah", "n15n", "n13c", "n18o", "nelec", "nfe",
]

# Special reaction indices (network.f90:263-265).
REACTION_PARAMS = [
    "nR_H2Form_CT", "nR_H2Form_ERDes", "nR_H2Form_ER", "nR_H2Form_LH",
    "nR_H2Form_LHDes", "nR_HFreeze", "nR_EFreeze", "nR_H2_hv", "nR_H2_crp",
    "nR_H2Freeze", "nR_C_hv", "nR_CO_hv",
]

# Term shapes of the generated RHS.  Each is a left-to-right product exactly as
# odes.f90 writes it; the evaluators reproduce the same operation order.
SHAPES = [
    "RATE*D*Y*Y",                    # 0  two-body gas phase
    "RATE*Y",                        # 1  one-body
    "RATE*D*Y",                      # 2  freeze-out / H2FORM single-H
    "RATE*Y/safeMantle",             # 3  desorption of surface species
    "RATE*Y*Y",                      # 4  LH on surface (density folded into rate)
    "RATE*Y*Y*bulkLayersReciprocal", # 5  LH in bulk
    "RATE*Y*bulkLayersReciprocal",   # 6  bulk swap / bulk photo
    "RATE*D*Y/safeMantle*Y",         # 7  DESOH2 (times Y(H))
    "RATE*Y*totalSwap/safeMantle",   # 8  surface swap
    "RATE*D*Y*Y/safeMantle",         # 9  Eley-Rideal
]
_SHAPE_RE = {
    0: r"RATE\((\d+)\)\*D\*Y\((\d+)\)\*Y\((\d+)\)$",
    1: r"RATE\((\d+)\)\*Y\((\d+)\)$",
    2: r"RATE\((\d+)\)\*D\*Y\((\d+)\)$",
    3: r"RATE\((\d+)\)\*Y\((\d+)\)/safeMantle$",
    4: r"RATE\((\d+)\)\*Y\((\d+)\)\*Y\((\d+)\)$",
    5: r"RATE\((\d+)\)\*Y\((\d+)\)\*Y\((\d+)\)\*bulkLayersReciprocal$",
    6: r"RATE\((\d+)\)\*Y\((\d+)\)\*bulkLayersReciprocal$",
    7: r"RATE\((\d+)\)\*D\*Y\((\d+)\)/safeMantle\*Y\((\d+)\)$",
    8: r"RATE\((\d+)\)\*Y\((\d+)\)\*totalSwap/safeMantle$",
    9: r"RATE\((\d+)\)\*D\*Y\((\d+)\)\*Y\((\d+)\)/safeMantle$",
}
_SHAPE_RE = {k: re.compile(v) for k, v in _SHAPE_RE.items()}
# number of density factors per shape (body count - 1 in MakeRates terms)
SHAPE_DPOW = np.array([1, 0, 1, 0, 0, 0, 0, 1, 0, 1], dtype=np.int32)
# modifier bits: 1 = /safeMantle, 2 = *bulkLayersReciprocal, 4 = *totalSwap
SHAPE_MOD = np.array([0, 0, 0, 1, 0, 2, 2, 1, 5, 1], dtype=np.int32)
MOD_SAFEMANTLE, MOD_BLR, MOD_TOTALSWAP = 1, 2, 4

_BLOB_MAGIC = b"UCLNET01"


def _join_continuations(src: str) -> str:
    return re.sub(r"&\s*\n\s*&", "", src)


def _parse_values(body: str) -> List[str]:
    out, cur, inq = [], [], False
    for ch in body:
        if ch == '"':
            inq = not inq
            cur.append(ch)
        elif ch == "," and not inq:
            out.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if cur:
        out.append("".join(cur).strip())
    return out


def _conv(v: str):
    vl = v.lower()
    if vl in (".true.", ".false."):
        return vl == ".true."
    if v.startswith('"'):
        return v.strip('"').strip()
    if re.fullmatch(r"[+-]?\d+", v):
        return int(v)
    return float(vl.replace("d", "e"))


def parse_network_f90(path: str) -> Dict[str, object]:
    """Parse the PARAMETER/variable arrays and scalar parameters of network.f90."""
    src = _join_continuations(open(path).read())
    arrays: Dict[str, object] = {}
    # array literals: NAME (N)=(/ ... /)
    for m in re.finditer(r"::\s*(\w+)\s*\((\d+)\)\s*=\s*\(/(.*?)/\)", src, re.S):
        name, n, body = m.group(1), int(m.group(2)), m.group(3)
        vals = [_conv(v) for v in _parse_values(body)]
        if len(vals) != n:
            raise ValueError(f"{name}: expected {n} values, got {len(vals)}")
        arrays[name] = vals
    # RESHAPE literal (garParams)
    m = re.search(r"garParams\((\d+),(\d+)\)\s*=\s*RESHAPE\(\(/(.*?)/\)", src, re.S)
    if m:
        nr, nc = int(m.group(1)), int(m.group(2))
        vals = [_conv(v) for v in _parse_values(m.group(3).replace(" ", ""))]
        # Fortran column-major (nr, nc)
        arrays["garParams"] = np.array(vals, dtype=np.float64).reshape(nc, nr).T
    # scalar integer parameters: name=value pairs in PARAMETER statements
    scalars: Dict[str, int] = {}
    for m in re.finditer(r"INTEGER\(dp\), PARAMETER ::\s*([^\n]*)", src):
        line = m.group(1)
        if "(" in line:
            continue
        for part in line.split(","):
            if "=" in part:
                k, v = part.split("=")
                scalars[k.strip()] = int(v.strip())
    arrays["_scalars"] = scalars
    m = re.search(r"THREE_PHASE\s*=\s*\.(\w+)\.", src)
    arrays["THREE_PHASE"] = bool(m and m.group(1).upper() == "TRUE")
    return arrays


def parse_odes_f90(path: str):
    """Parse the generated GETYDOT into ordered terms and the transfer branch."""
    src = _join_continuations(open(path).read())
    lines = [ln.strip() for ln in src.split("\n")]
    swap_terms: List[Tuple[int, int]] = []
    terms: List[Tuple[int, int, int, int, int, int]] = []
    pending = {}
    i = 0
    sums = {}
    transfer = {"neg": [], "pos": []}
    branch = None
    sum_expr = None
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("totalSwap="):
            for t in ln[len("totalSwap="):].split("+"):
                mm = _SHAPE_RE[6].match(t)
                if not mm:
                    raise ValueError("unexpected totalSwap term " + t)
                swap_terms.append((int(mm.group(1)) - 1, int(mm.group(2)) - 1))
        elif ln.startswith("LOSS = ") or (ln.startswith("PROD = RATE")):
            kind = "LOSS" if ln.startswith("LOSS") else "PROD"
            parsed = []
            for t in ln[7:].split("+"):
                for shape, rx in _SHAPE_RE.items():
                    mm = rx.match(t)
                    if mm:
                        g = [int(x) - 1 for x in mm.groups()]
                        ya = g[1]
                        yb = g[2] if len(g) > 2 else -1
                        parsed.append((g[0], shape, ya, yb))
                        break
                else:
                    raise ValueError("unrecognised term: " + t)
            pending[kind] = parsed
        elif ln.startswith("PROD = YDOT("):
            sum_expr = [int(x) - 1 for x in re.findall(r"YDOT\((\d+)\)", ln)]
        elif re.match(r"YDOT\((\d+)\) = PROD-LOSS$", ln):
            sp = int(re.match(r"YDOT\((\d+)\)", ln).group(1)) - 1
            for (r, shape, ya, yb) in pending["LOSS"]:
                terms.append((sp, -1, r, shape, ya, yb))
            for (r, shape, ya, yb) in pending["PROD"]:
                terms.append((sp, +1, r, shape, ya, yb))
            pending = {}
        elif re.match(r"YDOT\((\d+)\) = PROD$", ln):
            sp = int(re.match(r"YDOT\((\d+)\)", ln).group(1)) - 1
            sums.setdefault(sp, sum_expr)
        elif ln.startswith("IF (YDOT("):
            branch = "neg"
        elif ln == "ELSE":
            branch = "pos"
        elif ln == "ENDIF":
            branch = None
        elif branch and ln.startswith("YDOT("):
            mm = re.match(
                r"YDOT\((\d+)\)=YDOT\(\1\)([+-])YDOT\((\d+)\)\*surfaceCoverage\*Y\((\d+)\)(/safeBulk)?$",
                ln)
            if not mm:
                raise ValueError("unexpected transfer line " + ln)
            transfer[branch].append((int(mm.group(1)) - 1, 1 if mm.group(2) == "+" else -1,
                                     int(mm.group(4)) - 1, bool(mm.group(5))))
        i += 1
    return terms, swap_terms, sums, transfer


@dataclass
class Network:
    """Compiled network tables (all indices 0-based)."""
    nspec: int
    nreac: int
    species: List[str]
    mass: np.ndarray
    atom_counts: np.ndarray
    surface_list: np.ndarray
    bulk_list: np.ndarray
    ice_list: np.ndarray
    gas_ice_list: np.ndarray
    refractory_list: np.ndarray
    binding_energy: np.ndarray
    formation_enthalpy: np.ndarray
    three_phase: bool
    sp: Dict[str, int]          # named species, 0-based (absent -> nspec = density slot)
    rx: Dict[str, int]          # named reactions, 0-based
    re: np.ndarray              # (nreac, 3) reactants, -1 none
    pr: np.ndarray              # (nreac, 4) products, -1 none
    alpha: np.ndarray
    beta: np.ndarray
    gama: np.ndarray
    min_temps: np.ndarray
    max_temps: np.ndarray
    reduced_masses: np.ndarray
    extrapolate: np.ndarray
    freeze_partners: np.ndarray
    gar_params: np.ndarray      # (ngar, 7)
    ranges: Dict[str, Tuple[int, int]]  # Fortran 1-based inclusive (99999 = absent)
    terms: np.ndarray           # (nterm, 6): species, sign, rate, shape, ya, yb
    swap_terms: np.ndarray      # (nswap, 2): rate, y
    tr_surface: np.ndarray      # surface species of the transfer branch
    tr_bulk: np.ndarray         # matching bulk species
    # flux form (derived)
    flux_shape: np.ndarray = field(default=None)   # (nreac,) shape code, -1 if unused
    flux_ya: np.ndarray = field(default=None)
    flux_yb: np.ndarray = field(default=None)
    stoich_ptr: np.ndarray = field(default=None)   # CSR over species rows
    stoich_rx: np.ndarray = field(default=None)
    stoich_coef: np.ndarray = field(default=None)
    # linear invariants of the ODE system, [E, nspec] integer weights (None:
    # derived from the species names, see invariants())
    invariant_counts: np.ndarray = field(default=None)

    @property
    def neq(self) -> int:
        return self.nspec + 1

    def invariants(self) -> np.ndarray:
        """[E, nspec] integer weight vectors c with c . ydot = 0 for every
        reaction: the element counts (species-name counting of
        uclchem_gb300.analysis) of every element that each reaction conserves
        exactly.  An element that some reaction does not conserve (the
        default network's freeze-outs that hydrogenate, e.g. C2N -> #CH3CNH)
        is left out."""
        if self.invariant_counts is not None:
            return np.asarray(self.invariant_counts, dtype=np.int64).reshape(-1, self.nspec)
        from .analysis import ELEMENTS, element_counts
        S = np.zeros((self.nspec, self.nreac), dtype=np.int64)
        for i in range(self.nspec):
            for e in range(self.stoich_ptr[i], self.stoich_ptr[i + 1]):
                S[i, self.stoich_rx[e]] += self.stoich_coef[e]
        rows = []
        for el in ELEMENTS:
            if el in ("SURFACE", "BULK"):
                continue
            c = element_counts(self.species, el)
            if c.any() and not (c @ S).any():
                rows.append(c)
        return np.array(rows, dtype=np.int64).reshape(-1, self.nspec)

    # ------------------------------------------------------------------ #
    def derive_flux_form(self) -> None:
        """Regroup the generated terms per reaction and verify the regrouping.

        Every term of reaction r in odes.f90 must be the same product (same
        shape, same reactant slots up to order); the species-row coefficient
        is then the signed count of the reaction's terms in that row.
        """
        shape = -np.ones(self.nreac, dtype=np.int32)
        ya = -np.ones(self.nreac, dtype=np.int32)
        yb = -np.ones(self.nreac, dtype=np.int32)
        for (sp, sign, r, sh, a, b) in self.terms:
            key = (sh, tuple(sorted((a, b))) if b >= 0 else (a,))
            if shape[r] < 0:
                shape[r], ya[r], yb[r] = sh, a, b
            else:
                prev = (shape[r], tuple(sorted((ya[r], yb[r]))) if yb[r] >= 0 else (ya[r],))
                if prev != key:
                    raise ValueError(f"reaction {r+1} appears with two different products")
        for (r, y) in self.swap_terms:
            if shape[r] < 0:
                shape[r], ya[r], yb[r] = 6, y, -1
        coef: Dict[Tuple[int, int], int] = {}
        for (sp, sign, r, sh, a, b) in self.terms:
            coef[(sp, r)] = coef.get((sp, r), 0) + sign
        rows: List[List[Tuple[int, int]]] = [[] for _ in range(self.nspec)]
        for (sp, r), c in sorted(coef.items()):
            if c != 0:
                rows[sp].append((r, c))
        ptr = np.zeros(self.nspec + 1, dtype=np.int32)
        rxs, cfs = [], []
        for i, row in enumerate(rows):
            ptr[i + 1] = ptr[i] + len(row)
            for r, c in row:
                rxs.append(r)
                cfs.append(c)
        self.flux_shape, self.flux_ya, self.flux_yb = shape, ya, yb
        self.stoich_ptr = ptr
        self.stoich_rx = np.array(rxs, dtype=np.int32)
        self.stoich_coef = np.array(cfs, dtype=np.int32)

    # ------------------------------------------------------------------ #
    def save_npz(self, path: str) -> None:
        d = {k: v for k, v in self.__dict__.items() if isinstance(v, np.ndarray)}
        d["species"] = np.array(self.species)
        d["scalars"] = np.array([self.nspec, self.nreac, int(self.three_phase)], dtype=np.int64)
        d["sp_names"] = np.array(list(self.sp.keys()))
        d["sp_vals"] = np.array(list(self.sp.values()), dtype=np.int32)
        d["rx_names"] = np.array(list(self.rx.keys()))
        d["rx_vals"] = np.array(list(self.rx.values()), dtype=np.int32)
        d["range_names"] = np.array(list(self.ranges.keys()))
        d["range_vals"] = np.array(list(self.ranges.values()), dtype=np.int32)
        np.savez_compressed(path, **d)

    @classmethod
    def load_npz(cls, path: str) -> "Network":
        z = np.load(path, allow_pickle=False)
        nspec, nreac, three = (int(x) for x in z["scalars"])
        kw = {}
        for f in cls.__dataclass_fields__:
            if f in z.files and f != "species":
                kw[f] = z[f]
        net = cls(
            nspec=nspec, nreac=nreac, species=[str(s) for s in z["species"]],
            three_phase=bool(three),
            sp=dict(zip([str(s) for s in z["sp_names"]], [int(v) for v in z["sp_vals"]])),
            rx=dict(zip([str(s) for s in z["rx_names"]], [int(v) for v in z["rx_vals"]])),
            ranges=dict(zip([str(s) for s in z["range_names"]],
                            [tuple(int(x) for x in v) for v in z["range_vals"]])),
            **{k: v for k, v in kw.items() if k not in ("nspec", "nreac")},
        )
        return net

    # ------------------------------------------------------------------ #
    def to_blob(self) -> bytes:
        """Flat binary form read by the C ABI (``ucl_network_load``).

        Layout: magic ``UCLNET01``, then records of
        ``name[32] (NUL padded) | dtype u32 (1=i32, 2=f64) | count u64 | data``.
        """
        recs = []

        def add(name, arr, kind):
            arr = np.ascontiguousarray(arr, dtype=np.int32 if kind == 1 else np.float64).ravel()
            recs.append(struct.pack("<32sIQ", name.encode(), kind, arr.size) + arr.tobytes())

        add("dims", [self.nspec, self.nreac, int(self.three_phase)], 1)
        add("mass", self.mass, 2)
        add("atom_counts", self.atom_counts, 1)
        add("surface_list", self.surface_list, 1)
        add("bulk_list", self.bulk_list, 1)
        add("ice_list", self.ice_list, 1)
        add("gas_ice_list", self.gas_ice_list, 1)
        add("refractory_list", self.refractory_list, 1)
        add("binding_energy", self.binding_energy, 2)
        add("formation_enthalpy", self.formation_enthalpy, 2)
        add("sp", [self.sp[k] for k in SPECIES_PARAMS], 1)
        add("rx", [self.rx[k] for k in REACTION_PARAMS], 1)
        add("re", self.re, 1)
        add("pr", self.pr, 1)
        for k in ("alpha", "beta", "gama", "min_temps", "max_temps", "reduced_masses"):
            add(k, getattr(self, k), 2)
        add("extrapolate", self.extrapolate.astype(np.int32), 1)
        add("freeze_partners", self.freeze_partners, 1)
        add("gar_params", self.gar_params.reshape(-1, 7), 2)
        add("ranges", [self.ranges[k] for k in RANGE_NAMES], 1)
        add("terms", self.terms, 1)
        add("swap_terms", self.swap_terms, 1)
        add("tr_surface", self.tr_surface, 1)
        add("tr_bulk", self.tr_bulk, 1)
        add("flux_shape", self.flux_shape, 1)
        add("flux_ya", self.flux_ya, 1)
        add("flux_yb", self.flux_yb, 1)
        add("stoich_ptr", self.stoich_ptr, 1)
        add("stoich_rx", self.stoich_rx, 1)
        add("stoich_coef", self.stoich_coef, 1)
        # positive ions for enforceChargeConservation (chemistry.f90:114-121)
        add("ion_list", [i for i, name in enumerate(self.species) if "+" in name], 1)
        # linear invariants (conserved element counts), [E, nspec]
        add("inv_counts", self.invariants(), 1)
        return _BLOB_MAGIC + b"".join(recs)


def compile_network(network_f90: str, odes_f90: str) -> Network:
    """Compile MakeRates' network.f90 + odes.f90 into a :class:`Network`."""
    a = parse_network_f90(network_f90)
    terms, swap_terms, sums, transfer = parse_odes_f90(odes_f90)
    specname = a["specname"]
    nspec = len(specname)
    nreac = len(a["re1"])
    sc = a["_scalars"]

    def idx_list(name):
        return np.array([v - 1 for v in a[name]], dtype=np.int32)

    def rx_col(name):
        return np.array([v - 1 if 0 < v <= nspec else -1 for v in a[name]], dtype=np.int32)

    sp = {k: sc[k] - 1 for k in SPECIES_PARAMS}
    rx = {k: sc[k] - 1 for k in REACTION_PARAMS}
    ranges = {}
    src = _join_continuations(open(network_f90).read())
    for k in RANGE_NAMES:
        m = re.search(k + r"\s*\(2\)=\(/(\d+),(\d+)/\)", src)
        ranges[k] = (int(m.group(1)), int(m.group(2)))
    # transfer branch: both branches must be the standard surface/bulk pairing
    neg, pos = transfer["neg"], transfer["pos"]
    surf = np.array(a["surfaceList"], dtype=np.int32) - 1
    bulk = np.array(a["bulkList"], dtype=np.int32) - 1
    n = len(surf)
    exp_neg = [(int(surf[k]), -1, int(bulk[k]), True) for k in range(n)] + \
              [(int(bulk[k]), +1, int(bulk[k]), True) for k in range(n)]
    exp_pos = [(int(surf[k]), -1, int(surf[k]), False) for k in range(n)] + \
              [(int(bulk[k]), +1, int(surf[k]), False) for k in range(n)]
    if neg != exp_neg or pos != exp_pos:
        raise ValueError("transfer branch does not follow the surface/bulk pairing")
    nsurf_idx, nbulk_idx = sp["nsurface"], sp["nbulk"]
    if sorted(sums[nsurf_idx]) != sorted(surf.tolist()) or sorted(sums[nbulk_idx]) != sorted(bulk.tolist()):
        raise ValueError("BULK/SURFACE totals are not the surface/bulk list sums")
    refr = np.array([v - 1 for v in a["refractoryList"] if v > 0], dtype=np.int32)
    net = Network(
        nspec=nspec, nreac=nreac, species=[str(s) for s in specname],
        mass=np.array(a["mass"], dtype=np.float64),
        atom_counts=np.array(a["atomCounts"], dtype=np.int32),
        surface_list=surf, bulk_list=bulk,
        ice_list=idx_list("iceList"), gas_ice_list=idx_list("gasIceList"),
        refractory_list=refr,
        binding_energy=np.array(a["bindingEnergy"], dtype=np.float64),
        formation_enthalpy=np.array(a["formationEnthalpy"], dtype=np.float64),
        three_phase=a["THREE_PHASE"], sp=sp, rx=rx,
        re=np.stack([rx_col("re1"), rx_col("re2"), rx_col("re3")], axis=1),
        pr=np.stack([rx_col("p1"), rx_col("p2"), rx_col("p3"), rx_col("p4")], axis=1),
        alpha=np.array(a["alpha"], dtype=np.float64),
        beta=np.array(a["beta"], dtype=np.float64),
        gama=np.array(a["gama"], dtype=np.float64),
        min_temps=np.array(a["minTemps"], dtype=np.float64),
        max_temps=np.array(a["maxTemps"], dtype=np.float64),
        reduced_masses=np.array(a["reducedMasses"], dtype=np.float64),
        extrapolate=np.array(a["ExtrapolateRates"], dtype=bool),
        freeze_partners=idx_list("freezePartners"),
        gar_params=np.asarray(a["garParams"], dtype=np.float64).reshape(-1, 7),
        ranges=ranges,
        terms=np.array(terms, dtype=np.int32).reshape(-1, 6),
        swap_terms=np.array(swap_terms, dtype=np.int32).reshape(-1, 2),
        tr_surface=surf, tr_bulk=bulk,
    )
    net.derive_flux_form()
    return net


DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DEFAULT_NPZ = os.path.join(DATA_DIR, "default_network.npz")
DEFAULT_BLOB = os.path.join(DATA_DIR, "default_network.uclnet")


def load_default() -> Network:
    """The reference's default network (335 species, 3203 reactions), compiled."""
    return Network.load_npz(DEFAULT_NPZ)


def write_compiled(net: Network, npz_path: str, blob_path: str) -> None:
    net.save_npz(npz_path)
    with open(blob_path, "wb") as f:
        f.write(net.to_blob())


if __name__ == "__main__":  # MakeRates hook: python -m uclchem_gb300.network network.f90 odes.f90 [outdir]
    import sys
    nf, of = sys.argv[1], sys.argv[2]
    out = sys.argv[3] if len(sys.argv) > 3 else DATA_DIR
    os.makedirs(out, exist_ok=True)
    net = compile_network(nf, of)
    write_compiled(net, os.path.join(out, "default_network.npz"),
                   os.path.join(out, "default_network.uclnet"))
    print(f"compiled {net.nspec} species, {net.nreac} reactions, {len(net.terms)} terms, "
          f"{len(net.stoich_rx)} stoichiometric entries")
