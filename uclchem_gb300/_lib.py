"""ctypes binding of the C ABI (include/uclchem_gb300.h).

The library is built in-tree (uclchem_gb300/build.py).  There is no CPU
fallback: every entry point raises if the CUDA library cannot be loaded or
returns an error code.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build
from .params import ModelParams

_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class ModelStats(ctypes.Structure):
    _fields_ = [("nst", ctypes.c_int64), ("nfe", ctypes.c_int64), ("nje", ctypes.c_int64),
                ("nlu", ctypes.c_int64), ("nni", ctypes.c_int64), ("ncfn", ctypes.c_int64),
                ("netf", ctypes.c_int64), ("n_intervals", ctypes.c_int32), ("n_retries", ctypes.c_int32),
                ("solve_ms", ctypes.c_double), ("t_rates_ms", ctypes.c_double), ("t_rhs_ms", ctypes.c_double),
                ("t_jac_ms", ctypes.c_double), ("t_lu_ms", ctypes.c_double), ("t_solve_ms", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


STATS_DTYPE = np.dtype([(n, np.int64) for n in ("nst", "nfe", "nje", "nlu", "nni", "ncfn", "netf")] +
                       [("n_intervals", np.int32), ("n_retries", np.int32), ("solve_ms", np.float64),
                        ("t_rates_ms", np.float64), ("t_rhs_ms", np.float64), ("t_jac_ms", np.float64),
                        ("t_lu_ms", np.float64), ("t_solve_ms", np.float64), ("queue_ms", np.float64),
                        ("latency_ms", np.float64)])
assert STATS_DTYPE.itemsize == ctypes.sizeof(ModelStats)

PREC_FP64 = 0
PREC_MIXED = 1

EXPORTS = ["ucl_params_default", "ucl_network_load", "ucl_network_free", "ucl_network_nspec",
           "ucl_network_nreac", "ucl_ctx_create", "ucl_ctx_create_multi", "ucl_ctx_destroy", "ucl_ctx_nspec",
           "ucl_ctx_nreac", "ucl_rates_batch", "ucl_rhs_batch", "ucl_jac_batch", "ucl_solve_models",
           "ucl_solve_models_device", "ucl_solve_models_nets_device", "ucl_ctx_slots", "ucl_lu_factor_device",
           "ucl_serve_models_device", "ucl_server_open", "ucl_server_capacity", "ucl_server_submit",
           "ucl_server_poll", "ucl_server_take", "ucl_server_close", "ucl_lu_factor_device_static",
           "ucl_ctx_lu_variant"]

E_AGAIN = -107

_LOCK = threading.Lock()
_LIB = None


class UclError(RuntimeError):
    pass


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libuclchem_gb300.so (building it in-tree if needed)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if build_if_missing and (not os.path.exists(path) or _build.needs_build()):
            _build.build()
        if not os.path.exists(path):
            raise UclError("CUDA library not built: run uclchem_gb300.build.build()")
        lib = ctypes.CDLL(path)
        lib.ucl_params_default.argtypes = [ctypes.POINTER(ModelParams)]
        lib.ucl_network_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(_vp)]
        lib.ucl_network_free.argtypes = [_vp]
        lib.ucl_network_nspec.argtypes = [_vp]
        lib.ucl_network_nreac.argtypes = [_vp]
        lib.ucl_ctx_create.argtypes = [_vp, ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(_vp)]
        lib.ucl_ctx_create_multi.argtypes = [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, ctypes.c_size_t,
                                             ctypes.POINTER(_vp)]
        lib.ucl_ctx_destroy.argtypes = [_vp]
        lib.ucl_ctx_nspec.argtypes = [_vp]
        lib.ucl_ctx_nreac.argtypes = [_vp]
        lib.ucl_ctx_lu_variant.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                           ctypes.POINTER(ctypes.c_float)]
        lib.ucl_rates_batch.argtypes = [_vp, ctypes.c_int, _vp, _dp, _dp, _dp, _dp]
        lib.ucl_rhs_batch.argtypes = [_vp, ctypes.c_int, _vp, _dp, _dp, _dp, _dp]
        lib.ucl_jac_batch.argtypes = [_vp, ctypes.c_int, _vp, _dp, _dp, _dp, _dp]
        lib.ucl_solve_models.argtypes = [_vp, ctypes.c_int, _vp, _dp, ctypes.c_int, _dp, _dp, _ip, _ip, _vp,
                                         ctypes.c_int, _dp]
        lib.ucl_solve_models_device.argtypes = [_vp, ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp,
                                                ctypes.c_int, ctypes.c_int, _vp, _vp]
        lib.ucl_solve_models_nets_device.argtypes = [_vp, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, _vp, _vp, _vp,
                                                     _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]
        _llp = ctypes.POINTER(ctypes.c_longlong)
        lib.ucl_server_open.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.POINTER(_vp)]
        lib.ucl_server_capacity.argtypes = [_vp]
        lib.ucl_server_submit.argtypes = [_vp, _vp, _llp]
        lib.ucl_server_poll.argtypes = [_vp, ctypes.c_longlong]
        lib.ucl_server_take.argtypes = [_vp, ctypes.c_longlong, _dp, _dp, _ip, _ip, _vp]
        lib.ucl_server_close.argtypes = [_vp]
        lib.ucl_ctx_slots.argtypes = [_vp, ctypes.c_int]
        lib.ucl_lu_factor_device.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp]
        lib.ucl_lu_factor_device_static.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp]
        lib.ucl_serve_models_device.argtypes = [_vp, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, _vp, _vp, _vp, _vp,
                                                _vp, ctypes.c_int, ctypes.c_int, _vp]
        _LIB = lib
        return lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise UclError(f"{what} failed with code {rc}")


def _p(a):
    return a.ctypes.data_as(_dp)


class Context:
    """Loaded networks on one GPU (ucl_ctx).  `blob_path` is one network
    blob or a list of them (ucl_ctx_create_multi); per-model arrays use the
    strides of the largest network (nspec, neq, nreac below)."""

    def __init__(self, blob_path, device: int = 0, hbm_budget: int = 0):
        lib = load()
        self.lib = lib
        paths = [blob_path] if isinstance(blob_path, (str, bytes, os.PathLike)) else list(blob_path)
        self.nets = []
        for p in paths:
            net = _vp()
            check(lib.ucl_network_load(os.fsencode(p), ctypes.byref(net)), "ucl_network_load")
            self.nets.append(net)
        self.net = self.nets[0]
        self.net_nspec = [lib.ucl_network_nspec(n) for n in self.nets]
        self.net_nreac = [lib.ucl_network_nreac(n) for n in self.nets]
        ctx = _vp()
        if len(self.nets) == 1:
            check(lib.ucl_ctx_create(self.net, device, hbm_budget, ctypes.byref(ctx)), "ucl_ctx_create")
        else:
            arr = (_vp * len(self.nets))(*self.nets)
            check(lib.ucl_ctx_create_multi(arr, len(self.nets), device, hbm_budget, ctypes.byref(ctx)),
                  "ucl_ctx_create_multi")
        self.ctx = ctx
        self.nspec = lib.ucl_ctx_nspec(ctx)
        self.nreac = lib.ucl_ctx_nreac(ctx)
        self.neq = self.nspec + 1

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.ucl_ctx_destroy(self.ctx)
            self.ctx = None
        for n in getattr(self, "nets", []):
            self.lib.ucl_network_free(n)
        self.nets = []
        self.net = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def slots(self, precision: int) -> int:
        return self.lib.ucl_ctx_slots(self.ctx, precision)

    def lu_variant(self, net: int = 0):
        """(tensor_cores, us_tensor, us_cuda): the autotuner's FP32 LU choice
        for network `net` and its timings."""
        a, b = ctypes.c_float(0), ctypes.c_float(0)
        v = self.lib.ucl_ctx_lu_variant(self.ctx, net, ctypes.byref(a), ctypes.byref(b))
        if v < 0:
            raise UclError(f"ucl_ctx_lu_variant failed with code {v}")
        return bool(v), float(a.value), float(b.value)

    # ---------------------------------------------------------------- #
    def rates(self, params: np.ndarray, abund: np.ndarray, av: np.ndarray, phi: np.ndarray):
        n = len(params)
        ab = np.ascontiguousarray(abund, dtype=np.float64).reshape(n, self.neq).copy()
        av = np.ascontiguousarray(av, dtype=np.float64)
        ph = np.ascontiguousarray(phi, dtype=np.float64).copy()
        out = np.zeros((n, self.nreac))
        check(self.lib.ucl_rates_batch(self.ctx, n, params.ctypes.data, _p(ab), _p(av), _p(ph), _p(out)),
              "ucl_rates_batch")
        return out, ab, ph

    def rhs(self, params, y, rates, av):
        n = len(params)
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(n, self.neq)
        r = np.ascontiguousarray(rates, dtype=np.float64).reshape(n, self.nreac)
        av = np.ascontiguousarray(av, dtype=np.float64)
        out = np.zeros((n, self.neq))
        check(self.lib.ucl_rhs_batch(self.ctx, n, params.ctypes.data, _p(y), _p(r), _p(av), _p(out)),
              "ucl_rhs_batch")
        return out

    def jac(self, params, y, rates, av):
        n = len(params)
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(n, self.neq)
        r = np.ascontiguousarray(rates, dtype=np.float64).reshape(n, self.nreac)
        av = np.ascontiguousarray(av, dtype=np.float64)
        out = np.zeros((n, self.neq, self.neq))
        check(self.lib.ucl_jac_batch(self.ctx, n, params.ctypes.data, _p(y), _p(r), _p(av), _p(out)),
              "ucl_jac_batch")
        return out

    def solve_models(self, params: np.ndarray, max_rows: int, start=None, precision: int = PREC_MIXED,
                     rates: bool = False):
        """Whole models through ucl_solve_models (host buffers).  Returns
        (phys, abund, nrows, flags, stats), plus the rates rows when
        `rates` is set."""
        n = len(params)
        phys = np.zeros((n, max_rows, 8))
        ab = np.zeros((n, max_rows, self.nspec))
        nrows = np.zeros(n, dtype=np.int32)
        flags = np.zeros(n, dtype=np.int32)
        stats = np.zeros(n, dtype=STATS_DTYPE)
        rr = np.zeros((n, max_rows, self.nreac)) if rates else None
        st = None
        if start is not None:
            st = np.ascontiguousarray(start, dtype=np.float64).reshape(n, self.neq)
        check(self.lib.ucl_solve_models(self.ctx, n, params.ctypes.data, None if st is None else _p(st), max_rows,
                                        _p(phys), _p(ab), nrows.ctypes.data_as(_ip), flags.ctypes.data_as(_ip),
                                        stats.ctypes.data, precision, None if rr is None else _p(rr)),
              "ucl_solve_models")
        if rates:
            return phys, ab, nrows, flags, stats, rr
        return phys, ab, nrows, flags, stats

    def lu_factor_device(self, nsys, n, precision, mats_ptr, perm_ptr, info_ptr, stream=0):
        check(self.lib.ucl_lu_factor_device(self.ctx, nsys, n, precision, mats_ptr, perm_ptr, info_ptr, stream),
              "ucl_lu_factor_device")

    def serve_models_device(self, n, params_ptr, arrival_ptr, start_ptr, max_rows, phys_ptr, abund_ptr, nrows_ptr,
                            flags_ptr, stats_ptr, precision, max_ctas=0, stream=0):
        check(self.lib.ucl_serve_models_device(self.ctx, n, params_ptr, arrival_ptr, start_ptr, max_rows, phys_ptr,
                                               abund_ptr, nrows_ptr, flags_ptr, stats_ptr, precision, max_ctas,
                                               stream), "ucl_serve_models_device")

    def solve_models_device(self, n, params_ptr, start_ptr, max_rows, phys_ptr, abund_ptr, nrows_ptr, flags_ptr,
                            stats_ptr, precision, max_ctas=0, stream=0, rates_ptr=None):
        check(self.lib.ucl_solve_models_device(self.ctx, n, params_ptr, start_ptr, max_rows, phys_ptr, abund_ptr,
                                               nrows_ptr, flags_ptr, stats_ptr, precision, max_ctas, stream,
                                               rates_ptr), "ucl_solve_models_device")

    def solve_models_nets_device(self, n, net_of_ptr, params_ptr, start_ptr, max_rows, phys_ptr, abund_ptr,
                                 nrows_ptr, flags_ptr, stats_ptr, precision, max_ctas=0, stream=0, rates_ptr=None):
        check(self.lib.ucl_solve_models_nets_device(self.ctx, n, net_of_ptr, params_ptr, start_ptr, max_rows,
                                                    phys_ptr, abund_ptr, nrows_ptr, flags_ptr, stats_ptr, rates_ptr,
                                                    precision, max_ctas, stream), "ucl_solve_models_nets_device")


class Server:
    """A live serving session (ucl_server_*): submit requests while the
    persistent solver runs, poll them, take their outputs."""

    def __init__(self, ctx: Context, capacity: int, max_rows: int, precision: int = PREC_MIXED, max_ctas: int = 0,
                 idle_timeout_s: float = 0.0):
        self.ctx = ctx
        self.lib = ctx.lib
        self.max_rows = max_rows
        srv = _vp()
        check(self.lib.ucl_server_open(ctx.ctx, capacity, max_rows, precision, max_ctas, idle_timeout_s,
                                       ctypes.byref(srv)), "ucl_server_open")
        self.srv = srv
        self.capacity = self.lib.ucl_server_capacity(srv)

    def submit(self, param_record) -> int:
        """Queue one model (a PARAMS_DTYPE record); returns its request
        number, or None while the ring is full (take finished requests)."""
        k = ctypes.c_longlong(-1)
        rec = np.ascontiguousarray(param_record)
        rc = self.lib.ucl_server_submit(self.srv, rec.ctypes.data, ctypes.byref(k))
        if rc == E_AGAIN:
            return None
        check(rc, "ucl_server_submit")
        return int(k.value)

    def poll(self, k: int) -> bool:
        rc = self.lib.ucl_server_poll(self.srv, k)
        if rc < 0:
            raise UclError(f"ucl_server_poll failed with code {rc}")
        return rc == 1

    def take(self, k: int):
        phys = np.zeros((self.max_rows, 8))
        ab = np.zeros((self.max_rows, self.ctx.nspec))
        nr = np.zeros(1, dtype=np.int32)
        fl = np.zeros(1, dtype=np.int32)
        st = np.zeros(1, dtype=STATS_DTYPE)
        check(self.lib.ucl_server_take(self.srv, k, _p(phys), _p(ab), nr.ctypes.data_as(_ip), fl.ctypes.data_as(_ip),
                                       st.ctypes.data), "ucl_server_take")
        return phys, ab, int(nr[0]), int(fl[0]), st[0]

    def close(self):
        if getattr(self, "srv", None):
            rc = self.lib.ucl_server_close(self.srv)
            self.srv = None
            check(rc, "ucl_server_close")
