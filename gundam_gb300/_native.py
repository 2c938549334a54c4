"""ctypes bindings of libgw.so (include/gw.h) and libgw_workload.so (include/gw_workload.h).

The libraries are loaded from ``gundam_gb300/_lib``.  A missing library is an
error: there is no pure-Python or CPU fallback for the engine.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIBDIR = Path(__file__).resolve().parent / "_lib"

# status codes (gw.h)
GW_OK = 0
GW_ERR_ARG = 1
GW_ERR_STATE = 2
GW_ERR_CUDA = 3
GW_ERR_NOMEM = 4
GW_ERR_LIMIT = 5
GW_ERR_DEVICE_TIMEOUT = 6
GW_ERR_NOT_FINITE = 7

# dial types
GW_DIAL_NORM = 1
GW_DIAL_MONOTONIC = 2
GW_DIAL_UNIFORM = 3
GW_DIAL_GENERAL = 4
GW_DIAL_COMPACT = 5
GW_DIAL_GRAPH = 6
GW_DIAL_BILINEAR = 7
GW_DIAL_BICUBIC = 8
GW_DIAL_TABULATED = 9
GW_DIAL_KRIGED = 10

GW_FP64 = 0
GW_FP32 = 1
GW_DF64 = 2
GW_FLAG_SPLINE_KNOTS = 1
GW_FLAG_SPLINE_SLOPES = 2
GW_FLAG_SPLINE_COEFS = 3
GW_FLAG_SPLINE_GRID = 4

GW_LLH_NONE = 0
GW_LLH_POISSON = 1
GW_LLH_BARLOW_BEESTON_OA2021 = 2

GW_TABLE_FN_OSCILLATION = 1

# workload configurations (gw_workload.h)
GWW_C1 = 1
GWW_C2 = 2
GWW_C5 = 5
GWW_MIXED_SMALL = 9


class GwConfig(C.Structure):
    _fields_ = [
        ("n_results", C.c_int32),
        ("n_params", C.c_int32),
        ("n_bins", C.c_int32),
        ("k_max", C.c_int32),
        ("precision", C.c_int32),
        ("device", C.c_int32),
        ("tile_bytes", C.c_int32),
        ("flags", C.c_int32),
    ]


class GwLayoutInfo(C.Structure):
    _fields_ = [
        ("n_tiles", C.c_int64),
        ("n_dials", C.c_int64),
        ("payload_bytes", C.c_int64),
        ("header_bytes", C.c_int64),
        ("event_bytes", C.c_int64),
        ("partial_slots", C.c_int64),
        ("dials_by_type", C.c_int64 * 11),
    ]


class GwwWorkload(C.Structure):
    _fields_ = [
        ("config", C.c_int32),
        ("n_events", C.c_int32),
        ("n_params", C.c_int32),
        ("n_bins", C.c_int32),
        ("n_samples", C.c_int32),
        ("n_tables", C.c_int32),
        ("n_dials", C.c_int64),
        ("n_data", C.c_int64),
        ("max_weight", C.c_double),
        ("event_bin", C.POINTER(C.c_int32)),
        ("event_w0", C.POINTER(C.c_double)),
        ("event_dial_start", C.POINTER(C.c_int64)),
        ("dial_type", C.POINTER(C.c_uint8)),
        ("dial_par0", C.POINTER(C.c_int32)),
        ("dial_par1", C.POINTER(C.c_int32)),
        ("dial_data_start", C.POINTER(C.c_int64)),
        ("dial_data", C.POINTER(C.c_double)),
        ("mirror_lo", C.POINTER(C.c_double)),
        ("mirror_hi", C.POINTER(C.c_double)),
        ("clamp_lo", C.POINTER(C.c_double)),
        ("clamp_hi", C.POINTER(C.c_double)),
        ("truncate", C.POINTER(C.c_uint8)),
        ("prior_mean", C.POINTER(C.c_double)),
        ("prior_cov", C.POINTER(C.c_double)),
        ("sample_bin_start", C.POINTER(C.c_int32)),
        ("data", C.POINTER(C.c_double)),
        ("table_size", C.POINTER(C.c_int32)),
        ("table_fn_par", C.POINTER(C.c_int32)),
        ("table_node_start", C.POINTER(C.c_int64)),
        ("table_nodes", C.POINTER(C.c_double)),
        ("table_clamp", C.POINTER(C.c_double)),
    ]


_P = C.c_void_p
_I32 = C.c_int32
_I64 = C.c_int64
_D = C.c_double

# name -> argtypes for every gw_* entry point declared in include/gw.h
GW_SIGNATURES: dict[str, list] = {
    "gw_using_cuda": [_P],
    "gw_llh_bins": [_I32, _P, _P, _P, _I32, _P],
    "gw_has_gpu": [_P],
    "gw_create": [_P, _P],
    "gw_destroy": [_P],
    "gw_last_error": [_P, C.c_char_p, C.c_size_t],
    "gw_set_lower_mirror": [_P, _I32, _D],
    "gw_set_upper_mirror": [_P, _I32, _D],
    "gw_set_lower_clamp": [_P, _I32, _D],
    "gw_set_upper_clamp": [_P, _I32, _D],
    "gw_set_extrapolation": [_P, _I32, _I32],
    "gw_set_initial_value": [_P, _I32, _D],
    "gw_set_initial_values": [_P, _I32, _I32, _P],
    "gw_reserve_norm": [_P, _I32, _I32],
    "gw_add_spline": [_P, _I32, _I32, _I32, _P, _I32],
    "gw_add_graph": [_P, _I32, _I32, _P, _I32],
    "gw_add_surface": [_P, _I32, _I32, _I32, _I32, _P, _I32],
    "gw_add_tabulated": [_P, _I32, _I32, _I32, _D],
    "gw_add_kriged": [_P, _I32, _I32, _I32, _P, _P],
    "gw_add_dials": [_P, _I64, _P, _P, _P, _P, _P, _P],
    "gw_create_table": [_P, _I32, _P],
    "gw_set_table": [_P, _I32, _P, _I32],
    "gw_set_table_clamp": [_P, _I32, _D, _D],
    "gw_set_table_function": [_P, _I32, _I32, _P, _I32, _P, _I32],
    "gw_set_event_index": [_P, _I32, _I32],
    "gw_set_event_indices": [_P, _I32, _I32, _P],
    "gw_set_maximum_event_weight": [_P, _D],
    "gw_set_data": [_P, _P, _I32],
    "gw_set_likelihood": [_P, _I32],
    "gw_set_prior": [_P, _P, _P],
    "gw_add_eigen_block": [_P, _I32, _I32, _P],
    "gw_initialize": [_P],
    "gw_eval": [_P, _P, _I32, _P, _P, _P, _P],
    "gw_eval_device": [_P, _P, _I32, _P, _P, _P, _P, _P],
    "gw_sync": [_P],
    "gw_use_graph": [_P, _I32],
    "gw_autotune": [_P, _I32],
    "gw_get_shape": [_P, _P, _P, _P, _P],
    "gw_set_shape": [_P, _I32, _I32, _I32, _I32],
    "gw_set_shape_index": [_P, _I32],
    "gw_get_shape_index": [_P, _P],
    "gw_shape_count": [],
    "gw_shape_at": [_I32, _P, _P, _P, _P, _P, _P],
    "gw_set_plain_kernel": [_P, _I32],
    "gw_get_plain_kernel": [_P, _P],
    "gw_set_event_weight_copy": [_P, _I32],
    "gw_get_event_weights": [_P, _P],
    "gw_resident_memory": [_P, _P],
    "gw_get_layout": [_P, _P],
    "gw_set_profiling": [_P, _I32],
    "gw_llh_noalloc": [_P, _P, _P, _I32, _I32, _I32, _P, _P],
    "gw_selftest_wait_timeout": [C.c_uint32, _P],
    "gw_measure_fp32_peak": [_I32, _P],
    "gwm_create": [_P, _I32, _I32, _I32, _P],
    "gwm_destroy": [_P],
    "gwm_last_error": [_P, C.c_char_p, C.c_size_t],
    "gwm_set_layer": [_P, _I32, _P, _P],
    "gwm_get_layer": [_P, _I32, _P, _P],
    "gwm_forward": [_P, _P, _I32, _P, _I32],
    "gwm_train_step": [_P, _P, _P, _I32, C.c_float, _I32, _P],
    "gwm_gradients": [_P, _P, _P, _I32, _P, _P, _P],
    "gwm_gemm_test": [_P, _P, _I32, _I32, _I32, _P],
    "gwm_set_head": [_P, _P, _P, _P, _P, _P, _P, _P, _P],
    "gwm_predict": [_P, _P, _I32, _I32, _P, _P],
    "gwm_set_head_additive": [_P, _P, _P, _I32, C.c_float, _P, _P, _P, _P, _P, _P, _P],
    "gwm_set_chain": [_P, _P, _P, _P],
    "gwm_substeps": [_P, _P, _P, _I32, _I32, _I32, C.c_uint64, _P, _P, _P],
    "gwm_value_grad": [_P, _P, _I32, _I32, _P, _P],
    "gwm_train_reserve": [_P, C.c_int64],
    "gwm_train_size": [_P, _P],
    "gwm_train_append": [_P, _P, _P, _I32, _I32],
    "gwm_train_append_eval": [_P, _P, _P, _I32],
    "gwm_train_read": [_P, _I64, _I32, _P, _P],
    "gwm_train_epochs": [_P, _I32, _I32, C.c_float, C.c_float, C.c_uint64, _P],
    "gw_read_profile": [_P, _P, _P, _P],
}

GWW_SIGNATURES: dict[str, list] = {
    "gww_create": [_I32, _I64, C.c_uint64, _I32, _P],
    "gww_destroy": [_P],
    "gww_last_error": [],
}

_libs: dict[str, C.CDLL] = {}


def _load(name: str, sigs: dict[str, list]) -> C.CDLL:
    if name in _libs:
        return _libs[name]
    path = LIBDIR / name
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build the native libraries first "
            "(python -c 'import __graft_entry__ as g; g.build()')"
        )
    lib = C.CDLL(str(path))
    for fn, args in sigs.items():
        f = getattr(lib, fn)
        f.argtypes = args
        f.restype = C.c_int
    if name == "libgw_workload.so":
        lib.gww_last_error.restype = C.c_char_p
    _libs[name] = lib
    return lib


def libgw() -> C.CDLL:
    return _load("libgw.so", GW_SIGNATURES)


def libgw_workload() -> C.CDLL:
    return _load("libgw_workload.so", GWW_SIGNATURES)


class GwError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gw error {code}: {msg}")
        self.code = code


def last_error(engine_ptr) -> str:
    buf = C.create_string_buffer(1024)
    libgw().gw_last_error(engine_ptr, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, engine_ptr=None) -> None:
    if rc != GW_OK:
        raise GwError(rc, last_error(engine_ptr))
