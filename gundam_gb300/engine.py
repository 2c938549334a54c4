"""Python host side of the engine: a thin object over the C ABI in include/gw.h.

Method names follow the reference's operator API (Cache::Parameters,
Cache::Weights, the Cache::Weight::* calculators and Cache::HistogramSum,
src/CacheManager/include/*.h) so callers read like Cache::Manager::Update.
Every call goes through libgw.so; nothing here computes weights.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Engine:
    def __init__(self, n_results: int, n_params: int, n_bins: int, k_max: int = 1, precision: str = "fp64",
                 device: int = 0, tile_bytes: int = 0, spline_layout: str = "auto"):
        """spline_layout: stored form of the uniform-knot splines, "knots"
        (Catmull-Rom knot values, slopes formed on the device), "slopes"
        (slopes precomputed on the host), "coefs" (per-interval cubic
        coefficients, extrapolation intervals included), "grid" (the
        coefficients with the knot grid shared between splines, its interval
        formed once per point) or "auto" (knots for an FP32 engine with
        k_max == 1, grid for k_max >= 32 and for 16 <= k_max < 32 when the
        grid table holds at most 32 KB, else coefs for an FP64 engine with
        16 <= k_max < 32, slopes otherwise)."""
        self.lib = N.libgw()
        flags = {"auto": 0, "knots": N.GW_FLAG_SPLINE_KNOTS, "slopes": N.GW_FLAG_SPLINE_SLOPES,
                 "coefs": N.GW_FLAG_SPLINE_COEFS, "grid": N.GW_FLAG_SPLINE_GRID}[spline_layout]
        prec = {"fp32": N.GW_FP32, "fp64": N.GW_FP64, "df64": N.GW_DF64}[precision]
        cfg = N.GwConfig(int(n_results), int(n_params), int(n_bins), int(k_max), prec, int(device), int(tile_bytes),
                         flags)
        p = C.c_void_p()
        N.check(self.lib.gw_create(C.byref(cfg), C.byref(p)), None)
        self._e = p
        self.n_results, self.n_params, self.n_bins, self.k_max = n_results, n_params, n_bins, k_max
        self.precision = precision
        self._keep = []

    # ---- helpers ----
    def _chk(self, rc: int) -> None:
        N.check(rc, self._e)

    # ---- Cache::Parameters ----
    def set_lower_mirror(self, par, v): self._chk(self.lib.gw_set_lower_mirror(self._e, par, v))
    def set_upper_mirror(self, par, v): self._chk(self.lib.gw_set_upper_mirror(self._e, par, v))
    def set_lower_clamp(self, par, v): self._chk(self.lib.gw_set_lower_clamp(self._e, par, v))
    def set_upper_clamp(self, par, v): self._chk(self.lib.gw_set_upper_clamp(self._e, par, v))
    def set_extrapolation(self, par, allow): self._chk(self.lib.gw_set_extrapolation(self._e, par, int(allow)))

    # ---- Cache::Weights ----
    def set_initial_value(self, res, v): self._chk(self.lib.gw_set_initial_value(self._e, res, v))

    def set_initial_values(self, values, first=0):
        v = _c(values, np.float64)
        self._chk(self.lib.gw_set_initial_values(self._e, first, len(v), _ptr(v)))

    # ---- dial calculators ----
    def reserve_norm(self, res, par): self._chk(self.lib.gw_reserve_norm(self._e, res, par))

    def add_spline(self, dial_type, res, par, data):
        d = _c(data, np.float64)
        self._chk(self.lib.gw_add_spline(self._e, dial_type, res, par, _ptr(d), len(d)))

    def add_graph(self, res, par, data):
        d = _c(data, np.float64)
        self._chk(self.lib.gw_add_graph(self._e, res, par, _ptr(d), len(d)))

    def add_surface(self, dial_type, res, par1, par2, data):
        d = _c(data, np.float64)
        self._chk(self.lib.gw_add_surface(self._e, dial_type, res, par1, par2, _ptr(d), len(d)))

    def add_tabulated(self, res, table, index, fraction):
        self._chk(self.lib.gw_add_tabulated(self._e, res, table, index, fraction))

    def add_kriged(self, res, table, index, weight):
        i = _c(index, np.int32)
        w = _c(weight, np.float32)
        self._chk(self.lib.gw_add_kriged(self._e, res, table, len(i), _ptr(i), _ptr(w)))

    def add_dials(self, types, results, par0, par1, data_start, data):
        t, r = _c(types, np.uint8), _c(results, np.int32)
        p0, p1 = _c(par0, np.int32), _c(par1, np.int32)
        s, d = _c(data_start, np.int64), _c(data, np.float64)
        self._chk(self.lib.gw_add_dials(self._e, len(t), _ptr(t), _ptr(r), _ptr(p0), _ptr(p1), _ptr(s), _ptr(d)))

    # ---- tables ----
    def create_table(self, size) -> int:
        t = C.c_int32()
        self._chk(self.lib.gw_create_table(self._e, size, C.byref(t)))
        return t.value

    def set_table(self, table, values):
        v = _c(values, np.float64)
        self._chk(self.lib.gw_set_table(self._e, table, _ptr(v), len(v)))

    def set_table_clamp(self, table, lo, hi): self._chk(self.lib.gw_set_table_clamp(self._e, table, lo, hi))

    def set_table_function(self, table, params, nodes, fn=N.GW_TABLE_FN_OSCILLATION):
        p = _c(params, np.int32)
        n = _c(nodes, np.float64)
        self._chk(self.lib.gw_set_table_function(self._e, table, fn, _ptr(p), len(p), _ptr(n), len(n)))

    # ---- Cache::HistogramSum ----
    def set_event_index(self, res, b): self._chk(self.lib.gw_set_event_index(self._e, res, b))

    def set_event_indices(self, bins, first=0):
        b = _c(bins, np.int32)
        self._chk(self.lib.gw_set_event_indices(self._e, first, len(b), _ptr(b)))

    def set_maximum_event_weight(self, m): self._chk(self.lib.gw_set_maximum_event_weight(self._e, m))

    # ---- likelihood ----
    def set_data(self, data):
        d = _c(data, np.float64)
        self._chk(self.lib.gw_set_data(self._e, _ptr(d), len(d)))

    def set_likelihood(self, llh_type): self._chk(self.lib.gw_set_likelihood(self._e, llh_type))

    def set_prior(self, mean, icov):
        if mean is None:
            self._chk(self.lib.gw_set_prior(self._e, None, None))
            return
        m, ic = _c(mean, np.float64), _c(icov, np.float64)
        self._chk(self.lib.gw_set_prior(self._e, _ptr(m), _ptr(ic)))

    def add_eigen_block(self, first, V):
        V = _c(V, np.float64)
        self._keep.append(V)
        self._chk(self.lib.gw_add_eigen_block(self._e, int(first), V.shape[0], _ptr(V)))

    def initialize(self): self._chk(self.lib.gw_initialize(self._e))

    # ---- evaluation ----
    def eval(self, params: np.ndarray):
        """K points (K x n_params) -> (sums, sums2, llh, llh_stat)."""
        p = _c(np.atleast_2d(params), np.float64)
        K = p.shape[0]
        sums = np.empty((K, self.n_bins))
        sums2 = np.empty((K, self.n_bins))
        llh = np.empty(K)
        stat = np.empty(K)
        self._chk(self.lib.gw_eval(self._e, _ptr(p), K, _ptr(sums), _ptr(sums2), _ptr(llh), _ptr(stat)))
        return sums, sums2, llh, stat

    def eval_device(self, d_params: int, K: int, d_sums=0, d_sums2=0, d_llh=0, d_llh_stat=0, stream=0):
        """Device-pointer form (integers from e.g. torch's data_ptr()); asynchronous."""
        v = lambda x: C.c_void_p(x) if x else None  # noqa: E731
        self._chk(self.lib.gw_eval_device(self._e, v(d_params), K, v(d_sums), v(d_sums2), v(d_llh),
                                          v(d_llh_stat), v(stream)))

    def sync(self): self._chk(self.lib.gw_sync(self._e))
    def use_graph(self, on=True): self._chk(self.lib.gw_use_graph(self._e, int(on)))
    def autotune(self, K): self._chk(self.lib.gw_autotune(self._e, K))

    def shape(self):
        """(kernel family, points per pass, threads per block, payload stages) of the batched kernel;
        family 0 = k_batched (lanes over points), 1 = k_multi (threads over dials)."""
        k, a, b, c = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        self._chk(self.lib.gw_get_shape(self._e, C.byref(k), C.byref(a), C.byref(b), C.byref(c)))
        return k.value, a.value, b.value, c.value

    def set_shape(self, kind, points_per_pass, threads, stages):
        self._chk(self.lib.gw_set_shape(self._e, kind, points_per_pass, threads, stages))

    def set_shape_index(self, i):
        """Selects entry i of compiled_shapes()."""
        self._chk(self.lib.gw_set_shape_index(self._e, int(i)))

    def shape_index(self):
        """Entry of compiled_shapes() in use by the batched path."""
        i = C.c_int32()
        self._chk(self.lib.gw_get_shape_index(self._e, C.byref(i)))
        return i.value

    @staticmethod
    def compiled_shapes(lib=None):
        """Every compiled batched shape: (family, points per pass, points per
        thread, threads per block, payload stages, min CTAs per SM of its
        launch bounds (0: the compiler's choice))."""
        lib = lib or N.libgw()
        out = []
        v = [C.c_int32() for _ in range(6)]
        for i in range(lib.gw_shape_count()):
            N.check(lib.gw_shape_at(i, *[C.byref(x) for x in v]))
            out.append(tuple(x.value for x in v))
        return out

    def set_plain_kernel(self, kind): self._chk(self.lib.gw_set_plain_kernel(self._e, int(kind)))

    def plain_kernel(self) -> int:
        k = C.c_int32()
        self._chk(self.lib.gw_get_plain_kernel(self._e, C.byref(k)))
        return k.value

    def set_event_weight_copy(self, on=True): self._chk(self.lib.gw_set_event_weight_copy(self._e, int(on)))

    def event_weights(self) -> np.ndarray:
        w = np.empty(self.n_results)
        self._chk(self.lib.gw_get_event_weights(self._e, _ptr(w)))
        return w

    def resident_memory(self) -> int:
        b = C.c_int64()
        self._chk(self.lib.gw_resident_memory(self._e, C.byref(b)))
        return b.value

    def layout(self) -> dict:
        info = N.GwLayoutInfo()
        self._chk(self.lib.gw_get_layout(self._e, C.byref(info)))
        return {
            "n_tiles": info.n_tiles, "n_dials": info.n_dials, "payload_bytes": info.payload_bytes,
            "header_bytes": info.header_bytes, "event_bytes": info.event_bytes,
            "partial_slots": info.partial_slots, "dials_by_type": list(info.dials_by_type),
        }

    def set_profiling(self, on=True): self._chk(self.lib.gw_set_profiling(self._e, int(on)))

    def read_profile(self):
        """(weights-kernel ms summed, its launches, all engine kernel launches) since the last read."""
        ms, n, k = C.c_double(), C.c_int64(), C.c_int64()
        self._chk(self.lib.gw_read_profile(self._e, C.byref(ms), C.byref(n), C.byref(k)))
        return ms.value, n.value, k.value

    def close(self):
        if getattr(self, "_e", None):
            self.lib.gw_destroy(self._e)
            self._e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- convenience: load a generated workload ----
    @classmethod
    def from_workload(cls, wl, precision="fp64", k_max=1, llh_type=None, prior=True, device=0, tile_bytes=0,
                      per_dial=False, initialize=True, spline_layout="auto") -> "Engine":
        """Builds an engine holding `wl` the way Cache::Manager::Update fills its caches.

        per_dial=True issues one call per dial (the reference's AddSpline /
        AddGraph / ... sequence); otherwise one batched gw_add_dials call.
        initialize=False stops before gw_initialize (the engine holds its own
        copies by then, so a large workload can be released first)."""
        e = cls(wl.n_events, wl.n_params, wl.n_bins, k_max=k_max, precision=precision, device=device,
                tile_bytes=tile_bytes, spline_layout=spline_layout)
        for p in range(wl.n_params):
            if wl.mirror_lo[p] > -np.finfo(np.float64).max:
                e.set_lower_mirror(p, float(wl.mirror_lo[p]))
            if wl.mirror_hi[p] < np.finfo(np.float64).max:
                e.set_upper_mirror(p, float(wl.mirror_hi[p]))
            e.set_lower_clamp(p, float(wl.clamp_lo[p]))
            e.set_upper_clamp(p, float(wl.clamp_hi[p]))
            if wl.truncate[p]:
                e.set_extrapolation(p, False)
        for t in range(wl.n_tables):
            tid = e.create_table(int(wl.table_size[t]))
            assert tid == t
            e.set_table_clamp(t, float(wl.table_clamp[t, 0]), float(wl.table_clamp[t, 1]))
            nodes = wl.table_nodes[wl.table_node_start[t]:wl.table_node_start[t + 1]]
            if wl.table_fn_par[t, 0] >= 0:
                e.set_table_function(t, wl.table_fn_par[t], nodes)
            else:
                e.set_table(t, nodes)
        e.set_initial_values(wl.event_w0)
        e.set_event_indices(wl.event_bin)
        if wl.max_weight > 0:
            e.set_maximum_event_weight(wl.max_weight)
        res = wl.dial_result()
        if per_dial:
            _add_per_dial(e, wl, res)
        else:
            e.add_dials(wl.dial_type, res, wl.dial_par0, wl.dial_par1, wl.dial_data_start, wl.dial_data)
        e.set_data(wl.data)
        if llh_type is None:
            llh_type = N.GW_LLH_BARLOW_BEESTON_OA2021 if wl.config in (N.GWW_C2, N.GWW_C5) else N.GW_LLH_POISSON
        e.set_likelihood(llh_type)
        if prior:
            e.set_prior(wl.prior_mean, wl.prior_icov)
        if initialize:
            e.initialize()
        return e


def _add_per_dial(e: Engine, wl, res) -> None:
    for i in range(wl.n_dials):
        t = int(wl.dial_type[i])
        d = wl.dial_data[wl.dial_data_start[i]:wl.dial_data_start[i + 1]]
        r = int(res[i])
        p0 = int(wl.dial_par0[i])
        if t == N.GW_DIAL_NORM:
            e.reserve_norm(r, p0)
        elif t in (N.GW_DIAL_MONOTONIC, N.GW_DIAL_UNIFORM, N.GW_DIAL_GENERAL, N.GW_DIAL_COMPACT):
            e.add_spline(t, r, p0, d)
        elif t == N.GW_DIAL_GRAPH:
            e.add_graph(r, p0, d)
        elif t in (N.GW_DIAL_BILINEAR, N.GW_DIAL_BICUBIC):
            e.add_surface(t, r, p0, int(wl.dial_par1[i]), d)
        elif t == N.GW_DIAL_TABULATED:
            e.add_tabulated(r, int(d[0]), int(d[1]), float(d[2]))
        elif t == N.GW_DIAL_KRIGED:
            m = int(d[1])
            e.add_kriged(r, int(d[0]), d[2:2 + m].astype(np.int32), d[2 + m:2 + 2 * m].astype(np.float32))
        else:
            raise ValueError(f"unknown dial type {t}")
