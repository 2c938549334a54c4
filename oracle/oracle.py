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


REF_LLH = REF.parent / "libref_llh.so"
_ref_llh = None


def ref_llh_lib():
    """GUNDAM's own per-bin likelihood classes compiled for the host (only
    where oracle/_ref was built from the reference tree)."""
    global _ref_llh
    if _ref_llh is None and REF_LLH.exists():
        lib_ = C.CDLL(str(REF_LLH))
        lib_.ref_llh_bins.argtypes = [C.c_int32, _P, _P, _P, C.c_int32, _P, _P]
        lib_.ref_llh_bins.restype = C.c_int
        _ref_llh = lib_
    return _ref_llh


def ref_llh_bins(llh_type: int, data, pred, sqrt_sum_w2):
    """(values, threw) of the reference's per-bin likelihood; None without _ref."""
    lib_ = ref_llh_lib()
    if lib_ is None:
        return None
    d = np.ascontiguousarray(data, dtype=np.float64)
    p = np.ascontiguousarray(pred, dtype=np.float64)
    s = np.ascontiguousarray(sqrt_sum_w2, dtype=np.float64)
    out = np.empty(d.size)
    threw = np.zeros(d.size, dtype=np.int32)
    rc = lib_.ref_llh_bins(llh_type, d.ctypes.data, p.ctypes.data, s.ctypes.data, d.size, out.ctypes.data,
                           threw.ctypes.data)
    if rc != 0:
        raise RuntimeError("ref_llh_bins failed")
    return out, threw


REF_CACHE = REF.parent / "libref_cache.so"
_ref_cache = None


def ref_cache_lib():
    """GUNDAM's own Cache::Manager calculators compiled for the host (only
    where oracle/_ref was built from the reference tree)."""
    global _ref_cache
    if _ref_cache is None and REF_CACHE.exists():
        lib_ = C.CDLL(str(REF_CACHE), mode=C.RTLD_GLOBAL | os.RTLD_NOW)
        lib_.ref_cache_create.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int64] + [_P] * 13
        lib_.ref_cache_create.restype = C.c_int
        lib_.ref_cache_eval.argtypes = [_P, _P, _P, _P, _P]
        lib_.ref_cache_eval.restype = C.c_int
        lib_.ref_cache_error.argtypes = [_P]
        lib_.ref_cache_error.restype = C.c_char_p
        lib_.ref_cache_destroy.argtypes = [_P]
        lib_.ref_cache_destroy.restype = None
        _ref_cache = lib_
    return _ref_cache


class RefCache:
    """The reference's Cache::Weights + Cache::RecursiveSums filled from a
    Workload through its own operator API (oracle/ref/ref_cache.cpp)."""

    def __init__(self, wl):
        L = ref_cache_lib()
        if L is None:
            raise RuntimeError("oracle/_ref/libref_cache.so is not built")
        self.wl = wl
        self._keep = [np.ascontiguousarray(a) for a in (
            wl.dial_type, wl.dial_result(), wl.dial_par0, wl.dial_par1, wl.dial_data_start, wl.dial_data,
            wl.event_w0, wl.event_bin, wl.clamp_lo, wl.clamp_hi, wl.mirror_lo, wl.mirror_hi)]
        t, r, p0, p1, ds, d, w0, b, clo, chi, mlo, mhi = self._keep
        h = C.c_void_p()
        rc = L.ref_cache_create(wl.n_events, wl.n_params, wl.n_bins, wl.n_dials, _p(t), _p(r.astype(np.int32)),
                                _p(p0), _p(p1), _p(ds), _p(d), _p(w0), _p(b), _p(clo), _p(chi), _p(mlo), _p(mhi),
                                C.byref(h))
        if rc:
            raise RuntimeError(f"ref_cache_create: {L.ref_cache_error(None).decode()}")
        self._h = h

    def eval(self, params, weights=False):
        L = ref_cache_lib()
        p = np.ascontiguousarray(params, dtype=np.float64)
        s = np.empty(self.wl.n_bins)
        s2 = np.empty(self.wl.n_bins)
        w = np.empty(self.wl.n_events) if weights else None
        if L.ref_cache_eval(self._h, _p(p), _p(s), _p(s2), _p(w)):
            raise RuntimeError(f"ref_cache_eval: {L.ref_cache_error(self._h).decode()}")
        return (s, s2, w) if weights else (s, s2)

    def close(self):
        if getattr(self, "_h", None):
            ref_cache_lib().ref_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
