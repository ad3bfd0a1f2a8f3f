"""Element bookkeeping for conservation checks.

Restates the species-name element counting of the reference
(``src/uclchem/analysis.py:629-666``): an element's count in a species is the
number of occurrences of its symbol, plus ``i-1`` when the symbol is followed
by a digit ``i``, minus one for each longer element symbol that contains it
(``HE`` for ``H``, ``CL`` for ``C`` ...).  SURFACE and BULK totals are
excluded.
"""
from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

ELEMENTS = ["H", "D", "HE", "C", "N", "O", "F", "P", "S", "CL", "LI", "NA", "MG", "SI",
            "PAH", "15N", "13C", "18O", "SURFACE", "BULK"]


def element_counts(species: Sequence[str], element: str) -> np.ndarray:
    confusers = sorted([x for x in ELEMENTS if element in x and x != element], key=len, reverse=True)
    out = np.zeros(len(species), dtype=np.int64)
    for k, name in enumerate(species):
        s = name.count(element)
        for i in range(2, 10):
            if (element + str(i)) in name:
                s += i - 1
        for c in confusers:
            if c in name:
                s -= 1
        if name in ("SURFACE", "BULK"):
            s = 0
        out[k] = s
    return out


def element_matrix(species: Sequence[str], elements: Sequence[str] = ("H", "HE", "C", "N", "O", "S", "SI",
                                                                        "MG", "CL", "P", "F")) -> np.ndarray:
    return np.stack([element_counts(species, e) for e in elements])


def charge_vector(species: Sequence[str]) -> np.ndarray:
    """+1 per '+', -1 for the electron (charge bookkeeping of the network)."""
    q = np.zeros(len(species), dtype=np.int64)
    for k, name in enumerate(species):
        q[k] = name.count("+") - (1 if name == "E-" else 0)
    return q


def total_element_abundance(species: Sequence[str], abund: np.ndarray, element: str) -> np.ndarray:
    return np.asarray(abund)[..., :len(species)] @ element_counts(species, element)
