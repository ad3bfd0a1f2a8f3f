"""Python front end mirroring ``uclchem.model`` for the CLOUD, collapse and
hot-core models.

``cloud``, ``collapse`` and ``hot_core`` keep the signatures and return
layout of the reference's ``uclchem.model.cloud``, ``collapse`` and
``hot_core`` (src/uclchem/model.py:227-316, 319-426, 429-524): physics array ``[rows, points, 8]``,
abundance array ``[rows, points, nspec]``, rates, ``abundanceStart`` and the
success flag, with rows trimmed as ``_array_clean`` does (model.py:158-187).
The solve runs on the GPU through the C ABI; there is no CPU path.

``cloud_grid`` is the batched sibling: many parameter dictionaries in one
device launch, one persistent CTA per model, each with the cloud, a
collapse or the hot-core physics module.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

from . import network as _network
from ._lib import PREC_FP64, PREC_MIXED, Context, UclError
from .params import make_param_array, make_params

TIMEPOINTS = 500
N_PHYSICAL_PARAMETERS = 8
PHYSICAL_PARAMETERS = ["Time", "Density", "gasTemp", "dustTemp", "Av", "radfield", "zeta", "dstep"]

# the collapse argument of uclchem.model.collapse (model.py:355)
COLLAPSE_MODES = {"BE1.1": 1, "BE4": 2, "filament": 3, "ambipolar": 4}

_CTX: Optional[Context] = None


def get_context(device: int = 0) -> Context:
    """The process-wide context for the default network on `device`."""
    global _CTX
    if _CTX is None:
        _CTX = Context(_network.DEFAULT_BLOB, device=device)
    return _CTX


def _precision(p) -> int:
    if p in (PREC_FP64, PREC_MIXED):
        return p
    if isinstance(p, str) and p.lower() in ("fp64", "double", "plain"):
        return PREC_FP64
    if isinstance(p, str) and p.lower() in ("mixed", "fp32", "tc"):
        return PREC_MIXED
    raise ValueError(f"unknown precision {p!r}")


def _start_vectors(ctx: Context, params, starting_chemistry, n: int):
    if starting_chemistry is None:
        return None
    st = np.asarray(starting_chemistry, dtype=np.float64)
    if st.ndim == 1:
        st = np.broadcast_to(st, (n, st.shape[0]))
    out = np.zeros((n, ctx.neq))
    out[:, :min(st.shape[1], ctx.nspec)] = st[:, :ctx.nspec]
    # density slot: the value the reference holds there (initial density, or
    # 1.001x it for freefall, chemistry.f90:105 / cloud.f90:29)
    for i in range(n):
        d0 = params[i]["initialDens"]
        out[i, -1] = d0 * float(np.float32(1.001)) if params[i]["freefall"] else d0
    return out


def _collapse_mode(collapse) -> int:
    if isinstance(collapse, str):
        if collapse not in COLLAPSE_MODES:
            raise ValueError("collapse must be one of 'BE1.1', 'BE4', 'filament', or 'ambipolar'")
        return COLLAPSE_MODES[collapse]
    return int(collapse)


def cloud_grid(param_dicts: Sequence[Optional[dict]], timepoints: int = TIMEPOINTS,
               starting_chemistry=None, precision="mixed", context: Optional[Context] = None,
               return_rates: bool = False, collapse=0, hot_core=None):
    """Run many static/freefall CLOUD models in one device launch; with
    `collapse` (a mode name of COLLAPSE_MODES or its number, or one per
    model) the models run the collapse physics module instead, and with
    `hot_core` = (temp_indx, max_temperature) the hot-core module.

    Returns (physics [n, rows, 8], abundances [n, rows, nspec], nrows [n],
    flags [n], stats [n]) with rows = timepoints + 1, and the rates rows
    [n, rows, nreac] (the reference's ratesarray) when return_rates is set.
    """
    ctx = context or get_context()
    params = make_param_array(param_dicts)
    modes = collapse if isinstance(collapse, (list, tuple, np.ndarray)) else [collapse] * len(params)
    if len(modes) != len(params):
        raise ValueError("one collapse mode per parameter dictionary")
    params["collapse"] = [_collapse_mode(m) for m in modes]
    if hot_core is not None:
        params["hotcore"] = int(hot_core[0])
        params["maxTemperature"] = float(hot_core[1])
    start = _start_vectors(ctx, params, starting_chemistry, len(params))
    return ctx.solve_models(params, timepoints + 1, start=start, precision=_precision(precision),
                            rates=return_rates)


def cloud(param_dict=None, out_species: Optional[List[str]] = None, return_array: bool = False,
          return_dataframe: bool = False, return_rates: bool = False, starting_chemistry=None,
          timepoints: int = TIMEPOINTS, precision="mixed"):
    """Single CLOUD model with the reference's calling convention
    (pre_flight_checklist's argument rules, model.py:102-160)."""
    return _single(0, param_dict, out_species, return_array, return_dataframe, return_rates,
                   starting_chemistry, timepoints, precision)


def collapse(collapse, physics_output, param_dict=None, out_species: Optional[List[str]] = None,
             return_array: bool = False, return_dataframe: bool = False, return_rates: bool = False,
             starting_chemistry=None, timepoints: int = TIMEPOINTS, precision="mixed"):
    """Single collapse model (Priestley et al. 2018) with the reference's
    calling convention (model.py:319-426): `collapse` is 'BE1.1', 'BE4',
    'filament' or 'ambipolar'.  The reference's optional per-interval
    physics file (`physics_output`) is not written by the device path, so
    it must be None."""
    mode = _collapse_mode(collapse) if isinstance(collapse, str) else None
    if mode is None:
        raise ValueError("collapse must be one of 'BE1.1', 'BE4', 'filament', or 'ambipolar'")
    if physics_output is not None:
        raise ValueError("the device path does not write the collapse physics file: pass physics_output=None")
    return _single(mode, param_dict, out_species, return_array, return_dataframe, return_rates,
                   starting_chemistry, timepoints, precision)


def hot_core(temp_indx, max_temperature, param_dict=None, out_species: Optional[List[str]] = None,
             return_array: bool = False, return_dataframe: bool = False, return_rates: bool = False,
             starting_chemistry=None, timepoints: int = TIMEPOINTS, precision="mixed"):
    """Single hot-core model with the reference's calling convention
    (model.py:429-524): `temp_indx` 1-6 selects the protostar mass (1, 5,
    10, 15, 25, 60 Msun) of the temperature ramp, which stops rising at
    `max_temperature`."""
    return _single(0, param_dict, out_species, return_array, return_dataframe, return_rates,
                   starting_chemistry, timepoints, precision, hot_core=(temp_indx, max_temperature))


def _single(mode: int, param_dict, out_species, return_array, return_dataframe, return_rates,
            starting_chemistry, timepoints, precision, hot_core=None):
    if starting_chemistry is not None and not (return_array or return_dataframe):
        raise AssertionError("starting_chemistry can only be used with return_array or return_dataframe set to True")
    if return_rates and not (return_array or return_dataframe):
        raise AssertionError("return_rates can only be used with return_array or return_dataframe set to True")
    pd = dict(param_dict or {})
    file_keys = [k for k in pd if k.lower().endswith("file")]
    if file_keys:
        raise RuntimeError("file output is not part of the device path; offending keys: " + ", ".join(file_keys))
    ctx = get_context()
    try:
        make_params(pd)
    except ValueError:
        flag = -1
        if return_array or return_dataframe:
            return None, None, None, None, flag
        return [flag]
    out = cloud_grid([pd], timepoints=timepoints, starting_chemistry=starting_chemistry,
                     precision=precision, context=ctx, return_rates=return_rates, collapse=mode,
                     hot_core=hot_core)
    phys, ab, nrows, flags = out[:4]
    n = int(nrows[0])
    flag = int(flags[0])
    species = _network.load_default().species
    phys_a = phys[0, :n, None, :]
    chem_a = ab[0, :n, None, :]
    rates_a = out[5][0, :n, None, :] if return_rates else None
    abundance_start = ab[0, n - 1, :] if n > 0 else None
    if return_dataframe:
        import pandas as pd_  # not a dependency of the device path
        physics_df = pd_.DataFrame(phys_a[:, 0, :], columns=PHYSICAL_PARAMETERS)
        chem_df = pd_.DataFrame(chem_a[:, 0, :], columns=species)
        rates_df = pd_.DataFrame(rates_a[:, 0, :]) if return_rates else None
        return physics_df, chem_df, rates_df, abundance_start, flag
    if return_array:
        return phys_a, chem_a, rates_a, abundance_start, flag
    if flag < 0 or not out_species:
        return [flag]
    idx = [species.index(s) for s in out_species]
    return [flag] + [float(ab[0, n - 1, i]) for i in idx]
