"""ctypes front end of the CPU oracle (test infrastructure only).

Used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg to
check and time the GPU path against a CPU restatement of UCLCHEM's rates,
GETYDOT and DVODE (see ucl_oracle.c).  The product never imports this.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build
from uclchem_gb300 import network as _network
from uclchem_gb300.params import PARAMS_DTYPE, make_param_array, make_params

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


class Oracle:
    """One loaded network in the oracle."""

    def __init__(self, blob_path: Optional[str] = None):
        lib = ctypes.CDLL(_build.build())
        lib.orc_net_load.restype = _vp
        lib.orc_net_load.argtypes = [ctypes.c_char_p]
        lib.orc_net_free.argtypes = [_vp]
        lib.orc_net_set_ions.argtypes = [_vp, ctypes.c_int, _ip]
        lib.orc_cloud.restype = ctypes.c_int
        lib.orc_cloud.argtypes = [_vp, _vp, _dp, ctypes.c_int, _dp, _dp, _ip, _i64p]
        lib.orc_cloud_rates.restype = ctypes.c_int
        lib.orc_cloud_rates.argtypes = [_vp, _vp, _dp, ctypes.c_int, _dp, _dp, _ip, _i64p, _dp]
        lib.orc_cloud_batch.argtypes = [_vp, ctypes.c_int, _vp, _dp, ctypes.c_int, _dp, _dp, _ip, _ip, _i64p,
                                        ctypes.c_int]
        lib.orc_rates.argtypes = [_vp, _vp, _dp, ctypes.c_double, _dp, _dp]
        lib.orc_rhs.argtypes = [_vp, _vp, _dp, _dp, _dp, _dp]
        lib.orc_get_odes.argtypes = [_vp, _vp, _dp, _dp]
        lib.orc_fd_jacobian.argtypes = [_vp, _vp, _dp, _dp, _dp, ctypes.c_double, _dp]
        lib.orc_photo_rates.argtypes = [_vp, _vp, _dp, _dp]
        lib.orc_set_cpu_limit.argtypes = [ctypes.c_double]
        self.lib = lib
        path = blob_path or _network.DEFAULT_BLOB
        self.net = lib.orc_net_load(path.encode())
        if not self.net:
            raise RuntimeError(f"oracle could not load network {path}")
        self.tables = _network.Network.load_npz(path.replace(".uclnet", ".npz")) \
            if path.endswith(".uclnet") else None
        if self.tables is not None:
            ions = np.array([i for i, s in enumerate(self.tables.species) if "+" in s], dtype=np.int32)
            lib.orc_net_set_ions(self.net, len(ions), _ptr(ions, _ip))
        self.nspec = self.tables.nspec if self.tables is not None else None
        self.nreac = self.tables.nreac if self.tables is not None else None

    def __del__(self):
        try:
            self.lib.orc_net_free(self.net)
        except Exception:
            pass

    # ------------------------------------------------------------------ #
    CPU_LIMIT_FLAG = -99

    def set_cpu_limit(self, seconds: float) -> None:
        """Cap the CPU time of each later model of the calling thread: a
        model over the cap stops with flag CPU_LIMIT_FLAG (0 = no cap)."""
        self.lib.orc_set_cpu_limit(float(seconds))

    def cloud(self, param_dict=None, start=None, max_rows: int = 501, rates: bool = False):
        """One CLOUD model; returns (phys[rows,8], abund[rows,nspec], flag,
        counters), and the rates rows [rows, nreac] when `rates` is set."""
        p = np.array(param_dict, dtype=PARAMS_DTYPE) if isinstance(param_dict, (np.ndarray, np.void)) \
            else make_params(param_dict)
        phys = np.zeros((max_rows, 8))
        ab = np.zeros((max_rows, self.nspec))
        rr = np.zeros((max_rows, self.nreac)) if rates else None
        nrows = ctypes.c_int(0)
        cnt = np.zeros(9, dtype=np.int64)
        st = None if start is None else np.ascontiguousarray(start, dtype=np.float64)
        flag = self.lib.orc_cloud_rates(self.net, p.ctypes.data, None if st is None else _ptr(st), max_rows,
                                        _ptr(phys), _ptr(ab), ctypes.byref(nrows), _ptr(cnt, _i64p),
                                        None if rr is None else _ptr(rr))
        n = nrows.value
        if rates:
            return phys[:n], ab[:n], flag, cnt, rr[:n]
        return phys[:n], ab[:n], flag, cnt

    def cloud_batch(self, dicts: Sequence[dict], max_rows: int = 501, nthreads: int = 0):
        params = make_param_array(dicts)
        m = len(params)
        phys = np.zeros((m, max_rows, 8))
        ab = np.zeros((m, max_rows, self.nspec))
        nrows = np.zeros(m, dtype=np.int32)
        flags = np.zeros(m, dtype=np.int32)
        cnt = np.zeros((m, 9), dtype=np.int64)
        nthreads = nthreads or os.cpu_count() or 1
        self.lib.orc_cloud_batch(self.net, m, params.ctypes.data, None, max_rows, _ptr(phys), _ptr(ab),
                                 _ptr(nrows, _ip), _ptr(flags, _ip), _ptr(cnt, _i64p), nthreads)
        return phys, ab, nrows, flags, cnt

    def rates(self, param_dict, abund, phi=None):
        """Rates at the start of an interval; abund [neq] (surface/bulk totals refreshed)."""
        p = make_params(param_dict)
        ab = np.ascontiguousarray(abund, dtype=np.float64).copy()
        out = np.zeros(self.nreac)
        phys = np.zeros(4)
        phi = float(p["phi"]) if phi is None else float(phi)
        self.lib.orc_rates(self.net, p.ctypes.data, _ptr(ab), phi, _ptr(out), _ptr(phys))
        return out, ab, phys

    def rhs(self, param_dict, y, rates):
        p = make_params(param_dict)
        y = np.ascontiguousarray(y, dtype=np.float64)
        r = np.ascontiguousarray(rates, dtype=np.float64)
        ydot = np.zeros(self.nspec + 1)
        scale = np.zeros(self.nspec + 1)
        self.lib.orc_rhs(self.net, p.ctypes.data, _ptr(y), _ptr(r), _ptr(ydot), _ptr(scale))
        return ydot, scale

    def photo_rates(self, param_dict, y):
        """(H2, CO) photodissociation rates that F evaluates at state y."""
        p = make_params(param_dict)
        y = np.ascontiguousarray(y, dtype=np.float64)
        out = np.zeros(2)
        self.lib.orc_photo_rates(self.net, p.ctypes.data, _ptr(y), _ptr(out))
        return out

    def get_odes(self, param_dict, abund):
        p = make_params(param_dict)
        a = np.ascontiguousarray(abund, dtype=np.float64)
        ydot = np.zeros(self.nspec + 1)
        flag = self.lib.orc_get_odes(self.net, p.ctypes.data, _ptr(a), _ptr(ydot))
        return ydot, flag

    def fd_jacobian(self, param_dict, y, rates, ewt_inv, h):
        p = make_params(param_dict)
        n = self.nspec + 1
        jac = np.zeros(n * n)
        y = np.ascontiguousarray(y, dtype=np.float64)
        r = np.ascontiguousarray(rates, dtype=np.float64)
        w = np.ascontiguousarray(ewt_inv, dtype=np.float64)
        self.lib.orc_fd_jacobian(self.net, p.ctypes.data, _ptr(y), _ptr(r), _ptr(w), float(h), _ptr(jac))
        return jac.reshape(n, n).T  # row i, column j


def initial_abundances(oracle: Oracle, param_dict=None):
    """Elemental start vector (initializeChemistry) via a zero-length model."""
    d = dict(param_dict or {})
    d["finalTime"] = 0.0
    phys, ab, flag, _ = oracle.cloud(d, max_rows=2)
    return ab[0], phys[0]


class MassActionOracle:
    """The oracle's DVODE on a generic mass-action network (a
    uclchem_gb300.synthetic.SyntheticNetwork): flux_r = k_r y_a [n y_b]."""

    def __init__(self, net):
        lib = ctypes.CDLL(_build.build())
        args = [ctypes.c_int, ctypes.c_int, _ip, _ip, _dp, ctypes.c_double, _ip, _ip, _ip]
        lib.orc_ma_rhs.argtypes = args + [_dp, _dp]
        lib.orc_ma_solve.argtypes = args + [_dp, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_int, _dp, _i64p]
        lib.orc_ma_cloud.restype = ctypes.c_int
        lib.orc_ma_cloud.argtypes = args + [_dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp, _ip, _i64p]
        self.lib = lib
        self.net = net
        self._ra = np.ascontiguousarray(net.reactants[:, 0], dtype=np.int32)
        self._rb = np.ascontiguousarray(net.reactants[:, 1], dtype=np.int32)
        self._k = np.ascontiguousarray(net.k, dtype=np.float64)
        self._sptr = np.ascontiguousarray(net.stoich_ptr, dtype=np.int32)
        self._srx = np.ascontiguousarray(net.stoich_rx, dtype=np.int32)
        self._scoef = np.ascontiguousarray(net.stoich_coef, dtype=np.int32)

    def _common(self):
        return (self.net.nspec, self.net.nreac, _ptr(self._ra, _ip), _ptr(self._rb, _ip), _ptr(self._k),
                float(self.net.density), _ptr(self._sptr, _ip), _ptr(self._srx, _ip), _ptr(self._scoef, _ip))

    def rhs(self, y):
        y = np.ascontiguousarray(y, dtype=np.float64)
        out = np.zeros_like(y)
        self.lib.orc_ma_rhs(*self._common(), _ptr(y), _ptr(out))
        return out

    def solve(self, y0, tout, rtol=1e-8, atol_factor=1e-14, atol_min=1e-25, mxstep=100000):
        """Integrate from t = 0 through the output times tout (s).  Returns
        (abundances [len(tout), N], istate (0 = success), counters)."""
        y = np.array(y0, dtype=np.float64)
        tout = np.ascontiguousarray(tout, dtype=np.float64)
        yout = np.zeros((len(tout), len(y)))
        cnt = np.zeros(7, dtype=np.int64)
        rc = self.lib.orc_ma_solve(*self._common(), _ptr(y), len(tout), _ptr(tout), rtol, atol_factor, atol_min,
                                   mxstep, _ptr(yout), _ptr(cnt, _i64p))
        return yout, int(rc), cnt

    def cloud(self, y0, final_time_yr=1e6, rtol=1e-8, atol_factor=1e-14, atol_min=1e-25, mxstep=10000,
              max_rows=64):
        """The network integrated as the device integrates a generic network
        (orc_ma_cloud): density slot, CLOUD schedule to final_time_yr, retry
        and clamp logic.  Returns (times [rows] yr, abundances [rows, N],
        flag, counters)."""
        y0 = np.ascontiguousarray(y0, dtype=np.float64)[: self.net.nspec]
        yout = np.zeros((max_rows, self.net.nspec))
        tyr = np.zeros(max_rows)
        nrows = ctypes.c_int(0)
        cnt = np.zeros(9, dtype=np.int64)
        flag = self.lib.orc_ma_cloud(*self._common(), _ptr(y0), float(final_time_yr), rtol, atol_factor, atol_min,
                                     mxstep, max_rows, _ptr(yout), _ptr(tyr), ctypes.byref(nrows), _ptr(cnt, _i64p))
        r = nrows.value
        return tyr[:r], yout[:r], int(flag), cnt
