"""Model parameter dictionary: defaults, parsing and the C struct.

Mirrors UCLCHEM's parameter handling for the chemistry path:

* defaults of ``src/fortran_src/defaultparameters.f90:18-119``.  Fields the
  reference declares ``REAL(dp)`` but initialises from default-REAL literals
  (``rout=0.05``, ``fhe=0.1``, ``epsilon=0.01`` ...) carry the single-precision
  rounding of the literal, exactly as the compiled reference holds them;
* ``_reform_inputs`` lower-casing (``src/uclchem/model.py:47-73``);
* the key set and quirks of ``dictionaryParser`` (``wrap.f90:699-983``):
  unknown keys are an error (``PARAMETER_READ_ERROR``) and ``thermdesorb``
  sets ``uvdesorb`` (quirk Q2).
"""
from __future__ import annotations

import ctypes
from typing import Dict, Iterable, List, Optional

import numpy as np


def _sp(x: float) -> float:
    """Value of a Fortran default-REAL literal promoted to double."""
    return float(np.float32(x))


class ModelParams(ctypes.Structure):
    """ctypes mirror of ``ucl_model_params`` in include/uclchem_gb300.h."""
    _fields_ = [(n, ctypes.c_double) for n in (
        "initialTemp", "initialDens", "finalDens", "finalTime",
        "radfield", "zeta", "rout", "rin", "baseAv",
        "freezeFactor", "freefallFactor", "metallicity",
        "fh", "fhe", "fc", "fo", "fn", "fs", "fmg", "fsi", "fcl", "fp", "ff", "fd",
        "fli", "fna", "fpah", "f15n", "f13c", "f18o",
        "reltol", "abstol_factor", "abstol_min",
        "ebmaxh2", "ebmaxcr", "ebmaxuvcr", "epsilon", "uv_yield", "phi", "uvcreff", "omega",
    )] + [(n, ctypes.c_int32) for n in (
        "freefall", "endAtFinalDensity",
        "desorb", "h2desorb", "crdesorb", "uvdesorb", "thermdesorb",
        "ion", "points", "mxstep",
        "enforceChargeConservation", "improvedH2CRPDissociation",
        "cosmicRayAttenuation", "ionModel", "collapse", "hotcore",
    )] + [("maxTemperature", ctypes.c_double)]


PARAMS_DTYPE = np.dtype([(n, np.float64 if t is ctypes.c_double else np.int32)
                         for n, t in ModelParams._fields_])
assert PARAMS_DTYPE.itemsize == ctypes.sizeof(ModelParams)

# defaultparameters.f90:18-119 (single-precision literals rounded as compiled)
DEFAULTS: Dict[str, float] = {
    "initialTemp": _sp(10.0), "initialDens": 1.00e2, "finalDens": 1.00e5,
    "finalTime": 5.0e6, "radfield": _sp(1.0), "zeta": _sp(1.0),
    "rout": _sp(0.05), "rin": _sp(0.0), "baseAv": _sp(2.0),
    "freezeFactor": _sp(1.0), "freefallFactor": _sp(1.0), "metallicity": _sp(1.0),
    "fh": _sp(0.5), "fhe": _sp(0.1), "fc": 1.77e-04, "fo": 3.34e-04, "fn": 6.18e-05,
    "fs": 3.51e-6, "fmg": 2.256e-06, "fsi": 1.78e-06, "fcl": 3.39e-08,
    "fp": 7.78e-08, "ff": 3.6e-08, "fd": _sp(0.0), "fli": _sp(0.0), "fna": _sp(0.0),
    "fpah": _sp(0.0), "f15n": _sp(0.0), "f13c": _sp(0.0), "f18o": _sp(0.0),
    "reltol": 1e-8, "abstol_factor": 1.0e-14, "abstol_min": 1.0e-25,
    "ebmaxh2": 1.21e3, "ebmaxcr": 1.21e3, "ebmaxuvcr": 1.0e4,
    "epsilon": _sp(0.01), "uv_yield": _sp(0.03), "phi": 1.0e5, "uvcreff": 1.0e-3,
    "omega": _sp(0.5),
    "freefall": 0, "endAtFinalDensity": 0, "desorb": 1, "h2desorb": 1, "crdesorb": 1,
    "uvdesorb": 1, "thermdesorb": 1, "ion": 2, "points": 1, "mxstep": 10000,
    "enforceChargeConservation": 0, "improvedH2CRPDissociation": 0,
    "cosmicRayAttenuation": 0, "ionModel": ord("L"),
    # physics module (not dictionary keys: the collapse argument of
    # model.collapse, the temp_indx and max_temperature of model.hot_core;
    # 0 = cloud)
    "collapse": 0, "hotcore": 0, "maxTemperature": 0.0,
}

# dictionaryParser keys (lower case) -> struct field (wrap.f90:755-975)
_KEYMAP = {k.lower(): k for k in DEFAULTS}
_KEYMAP["thermdesorb"] = "uvdesorb"        # quirk Q2 (wrap.f90:802-803)
# accepted keys that do not reach the chemistry path
_IGNORED = {"outspecies", "writestep", "abundsavefile", "abundloadfile", "outputfile",
            "ratefile", "fluxfile", "columnfile", "ntime", "bm0", "instantsublimation",
            "currenttime"}
# module variables and struct fields without a dict key
_NOT_PARSED = {"mxstep", "enforcechargeconservation", "collapse", "hotcore", "maxtemperature"}


class ParameterError(ValueError):
    """Unknown or ill-typed parameter (reference code PARAMETER_READ_ERROR)."""


def _to_bool(v) -> int:
    if isinstance(v, str):
        s = v.strip().lower().strip(".")
        if s in ("true", "t"):
            return 1
        if s in ("false", "f"):
            return 0
        raise ParameterError(f"not a logical: {v!r}")
    return int(bool(v))


def _to_char(v) -> int:
    """A Fortran CHARACTER(1) read of the value: its first character (list-
    directed READ strips the surrounding quotes), as a character code."""
    s = str(v).strip().strip("'\"")
    if not s:
        raise ParameterError(f"not a character: {v!r}")
    return ord(s[0])


def make_params(param_dict: Optional[dict] = None) -> np.ndarray:
    """One ``ucl_model_params`` record from a UCLCHEM parameter dictionary."""
    rec = np.zeros((), dtype=PARAMS_DTYPE)
    for k, v in DEFAULTS.items():
        rec[k] = v
    if param_dict:
        lowered = {}
        for k, v in param_dict.items():
            lk = k.lower()
            if lk in lowered:
                raise ParameterError(f"Lower case key {k} is already in the dict")
            lowered[lk] = v
        for lk, v in lowered.items():
            if lk in _IGNORED:
                continue
            if lk in ("alpha", "beta", "gamma"):
                raise ParameterError("per-reaction coefficient overrides change the network tables; "
                                     "compile a modified network instead")
            if lk not in _KEYMAP or lk in _NOT_PARSED:
                raise ParameterError(f"Problem with given parameter: '{lk}'")
            field = _KEYMAP[lk]
            kind = PARAMS_DTYPE[field]
            try:
                if field == "ionModel":
                    rec[field] = _to_char(v)
                elif kind == np.int32:
                    rec[field] = _to_bool(v) if field not in ("ion", "points") else int(v)
                else:
                    rec[field] = float(v)
            except (TypeError, ValueError) as e:
                raise ParameterError(f"Error reading {lk}: {e}") from None
    return rec


def make_param_array(dicts: Iterable[Optional[dict]]) -> np.ndarray:
    dicts = list(dicts)
    arr = np.zeros(len(dicts), dtype=PARAMS_DTYPE)
    for i, d in enumerate(dicts):
        arr[i] = make_params(d)
    return arr


def stratified_sample(dicts: List[dict], size: int, seed: int = 20261203) -> List[int]:
    """Indices of a seeded sample of `size` grid points stratified over
    density: the points are ranked by initialDens, cut into `size` strata of
    equal count, and one point is drawn from each stratum (density is what
    the cost of a model grows with most)."""
    n = len(dicts)
    size = min(size, n)
    if size <= 0:
        return []
    order = np.argsort(np.array([d["initialDens"] for d in dicts]), kind="stable")
    rng = np.random.default_rng(seed + 1)
    out = []
    for k in range(size):
        lo, hi = k * n // size, (k + 1) * n // size
        out.append(int(order[lo + int(rng.integers(hi - lo))]))
    return out


def grid_params(n: int, seed: int = 20261203, final_time: float = 1.0e6,
                extra: Optional[dict] = None) -> List[dict]:
    """The 4096-point CLOUD grid of the benchmark: seeded log-uniform density
    1e2-1e7 cm^-3, uniform temperature 10-50 K, log-uniform zeta and radfield
    1-1e3, final time 1e6 yr."""
    rng = np.random.default_rng(seed)
    dens = 10.0 ** rng.uniform(2.0, 7.0, n)
    temp = rng.uniform(10.0, 50.0, n)
    zeta = 10.0 ** rng.uniform(0.0, 3.0, n)
    rad = 10.0 ** rng.uniform(0.0, 3.0, n)
    out = []
    for i in range(n):
        d = {"initialDens": float(dens[i]), "initialTemp": float(temp[i]),
             "zeta": float(zeta[i]), "radfield": float(rad[i]),
             "finalTime": final_time, "freefall": False, "endAtFinalDensity": False}
        if extra:
            d.update(extra)
        out.append(d)
    return out
