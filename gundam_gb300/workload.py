"""Synthetic workloads (libgw_workload.so) as numpy views.

A :class:`Workload` holds, in event-major order, what GUNDAM's
EventDialCache holds after DataDispenser::load: per event its global bin,
base weight and list of dials, each with the data vector its
DialBase::getDialData() returns; plus parameter metadata, the data
histogram and the prior.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

CONFIGS = {"c1": N.GWW_C1, "c2": N.GWW_C2, "c5": N.GWW_C5, "mixed": N.GWW_MIXED_SMALL}


def _view(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(int(n),)).view(dtype)


class Workload:
    """Owns one generated workload; arrays are zero-copy views of native memory."""

    def __init__(self, config: str | int, n_events: int = 0, seed: int = 1, threads: int = 0):
        cfg = CONFIGS[config] if isinstance(config, str) else int(config)
        lib = N.libgw_workload()
        p = C.c_void_p()
        rc = lib.gww_create(cfg, int(n_events), C.c_uint64(seed), int(threads), C.byref(p))
        if rc != 0:
            raise N.GwError(rc, lib.gww_last_error().decode())
        self._ptr = p
        w = C.cast(p, C.POINTER(N.GwwWorkload)).contents
        self._w = w
        self.config = cfg
        self.seed = seed
        self.n_events = w.n_events
        self.n_params = w.n_params
        self.n_bins = w.n_bins
        self.n_samples = w.n_samples
        self.n_tables = w.n_tables
        self.n_dials = w.n_dials
        self.n_data = w.n_data
        self.max_weight = w.max_weight
        E, D, P, B, T = self.n_events, self.n_dials, self.n_params, self.n_bins, self.n_tables
        self.event_bin = _view(w.event_bin, E, np.int32)
        self.event_w0 = _view(w.event_w0, E, np.float64)
        self.event_dial_start = _view(w.event_dial_start, E + 1, np.int64)
        self.dial_type = _view(w.dial_type, D, np.uint8)
        self.dial_par0 = _view(w.dial_par0, D, np.int32)
        self.dial_par1 = _view(w.dial_par1, D, np.int32)
        self.dial_data_start = _view(w.dial_data_start, D + 1, np.int64)
        self.dial_data = _view(w.dial_data, self.n_data, np.float64)
        self.mirror_lo = _view(w.mirror_lo, P, np.float64)
        self.mirror_hi = _view(w.mirror_hi, P, np.float64)
        self.clamp_lo = _view(w.clamp_lo, P, np.float64)
        self.clamp_hi = _view(w.clamp_hi, P, np.float64)
        self.truncate = _view(w.truncate, P, np.uint8)
        self.prior_mean = _view(w.prior_mean, P, np.float64)
        self.prior_cov = _view(w.prior_cov, P * P, np.float64).reshape(P, P)
        self.sample_bin_start = _view(w.sample_bin_start, self.n_samples + 1, np.int32)
        self.data = _view(w.data, B, np.float64)
        self.table_size = _view(w.table_size, T, np.int32)
        self.table_fn_par = _view(w.table_fn_par, 6 * T, np.int32).reshape(T, 6)
        self.table_node_start = _view(w.table_node_start, T + 1, np.int64)
        n_nodes = int(self.table_node_start[-1]) if T else 0
        self.table_nodes = _view(w.table_nodes, n_nodes, np.float64)
        self.table_clamp = _view(w.table_clamp, 2 * T, np.float64).reshape(T, 2) if T else np.zeros((0, 2))
        self._icov = None
        self._chol = None

    # the event -> dial map of every dial (dials are stored event-major)
    def dial_result(self) -> np.ndarray:
        counts = np.diff(self.event_dial_start)
        return np.repeat(np.arange(self.n_events, dtype=np.int32), counts)

    @property
    def prior_icov(self) -> np.ndarray:
        if self._icov is None:
            self._icov = np.ascontiguousarray(np.linalg.inv(self.prior_cov))
        return self._icov

    @property
    def prior_chol(self) -> np.ndarray:
        if self._chol is None:
            self._chol = np.linalg.cholesky(self.prior_cov)
        return self._chol

    def draw_points(self, k: int, seed: int, inflate: float = 1.0) -> np.ndarray:
        """k parameter points from the prior (covariance scaled by inflate**2)."""
        rng = np.random.default_rng(seed)
        z = rng.standard_normal((k, self.n_params))
        return np.ascontiguousarray(self.prior_mean[None, :] + inflate * z @ self.prior_chol.T)

    def nominal(self) -> np.ndarray:
        return np.ascontiguousarray(self.prior_mean[None, :].copy())

    def close(self) -> None:
        if getattr(self, "_ptr", None):
            N.libgw_workload().gww_destroy(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
