"""ctypes front end of liboracle.so (oracle.h) -- TEST INFRASTRUCTURE.

Used by tests, the smoke check and the benchmark's CPU-baseline leg only.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF = HERE / "_ref" / "libref_dials.so"

_P = C.c_void_p


class OracleInput(C.Structure):
    _fields_ = [
        ("n_events", C.c_int32), ("n_params", C.c_int32), ("n_bins", C.c_int32), ("n_samples", C.c_int32),
        ("n_tables", C.c_int32), ("llh_type", C.c_int32), ("max_weight", C.c_double),
        ("event_bin", _P), ("event_w0", _P), ("event_dial_start", _P), ("dial_type", _P), ("dial_par0", _P),
        ("dial_par1", _P), ("dial_data_start", _P), ("dial_data", _P), ("mirror_lo", _P), ("mirror_hi", _P),
        ("clamp_lo", _P), ("clamp_hi", _P), ("truncate", _P), ("sample_bin_start", _P), ("data", _P),
        ("table_size", _P), ("table_fn_par", _P), ("table_node_start", _P), ("table_nodes", _P),
        ("table_clamp", _P), ("prior_mean", _P), ("prior_icov", _P),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} missing: run the build first")
        _lib = C.CDLL(str(LIB))
        _lib.oracle_create.argtypes = [_P, _P]
        _lib.oracle_destroy.argtypes = [_P]
        _lib.oracle_eval.argtypes = [_P, _P, C.c_int32, C.c_int32, _P, _P, _P, _P, _P]
        _lib.oracle_dial.argtypes = [C.c_int32, _P, C.c_int32, C.c_double, C.c_double, C.c_int32]
        _lib.oracle_dial.restype = C.c_double
        _lib.oracle_llh_bin.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_double]
        _lib.oracle_llh_bin.restype = C.c_double
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """FP64 CPU propagation of a Workload (same inputs the engine receives)."""

    def __init__(self, wl, llh_type: int, prior: bool = True):
        self.wl = wl
        self._icov = np.ascontiguousarray(wl.prior_icov) if prior else None
        self._keep = [self._icov]
        inp = OracleInput()
        inp.n_events, inp.n_params, inp.n_bins = wl.n_events, wl.n_params, wl.n_bins
        inp.n_samples, inp.n_tables, inp.llh_type = wl.n_samples, wl.n_tables, llh_type
        inp.max_weight = wl.max_weight
        for name in ("event_bin", "event_w0", "event_dial_start", "dial_type", "dial_par0", "dial_par1",
                     "dial_data_start", "dial_data", "mirror_lo", "mirror_hi", "clamp_lo", "clamp_hi",
                     "truncate", "sample_bin_start", "data", "table_size", "table_fn_par", "table_node_start",
                     "table_nodes", "table_clamp"):
            arr = np.ascontiguousarray(getattr(wl, name))
            self._keep.append(arr)
            setattr(inp, name, _p(arr))
        inp.prior_mean = _p(wl.prior_mean) if prior else None
        inp.prior_icov = _p(self._icov) if prior else None
        self._inp = inp
        h = C.c_void_p()
        rc = lib().oracle_create(C.byref(inp), C.byref(h))
        if rc:
            raise RuntimeError(f"oracle_create failed ({rc})")
        self._h = h
        self.n_bins = wl.n_bins

    def eval(self, params, threads: int = 0, weights: bool = False):
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        K = p.shape[0]
        threads = threads or (os.cpu_count() or 1)
        sums = np.empty((K, self.n_bins))
        sums2 = np.empty((K, self.n_bins))
        stat = np.empty(K)
        pen = np.empty(K)
        w = np.empty(self.wl.n_events) if weights else None
        rc = lib().oracle_eval(self._h, _p(p), K, threads, _p(sums), _p(sums2), _p(stat), _p(pen), _p(w))
        if rc:
            raise RuntimeError(f"oracle_eval failed ({rc})")
        out = {"sums": sums, "sums2": sums2, "llh_stat": stat, "penalty": pen, "llh": stat + pen}
        if weights:
            out["weights"] = w
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dial(dial_type: int, data, x: float, y: float = 0.0, truncate: bool = False) -> float:
    d = np.ascontiguousarray(data, dtype=np.float64)
    return lib().oracle_dial(dial_type, _p(d), len(d), x, y, int(truncate))


def llh_bin(llh_type: int, data: float, pred: float, sqrt_sum_w2: float) -> float:
    return lib().oracle_llh_bin(llh_type, data, pred, sqrt_sum_w2)


_ref = None


def ref_lib():
    """The reference's own Calculate*.h functions (only where oracle/_ref was built)."""
    global _ref
    if _ref is None and REF.exists():
        _ref = C.CDLL(str(REF))
        for fn in ("ref_monotonic", "ref_compact", "ref_uniform", "ref_general", "ref_graph"):
            f = getattr(_ref, fn)
            f.argtypes = [C.c_double, C.c_double, C.c_double, _P, C.c_int]
            f.restype = C.c_double
        for fn in ("ref_bilinear", "ref_bicubic"):
            f = getattr(_ref, fn)
            f.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, _P, C.c_int]
            f.restype = C.c_double
    return _ref
