"""The C ABI: every symbol declared in include/*.h is exported, and the
builder rejects bad input before touching a device (CPU only)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from gundam_gb300 import Engine
from gundam_gb300 import _native as N

ROOT = Path(__file__).resolve().parents[1]


def _declared(header: str, prefix: str):
    text = (ROOT / "include" / header).read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(%s\w+)\s*\(" % prefix, text, re.M)))


def test_every_engine_symbol_is_exported_and_bound():
    names = _declared("gw.h", "gw")
    assert len(names) >= 40
    lib = N.libgw()
    for n in names:
        assert hasattr(lib, n), n
        assert n in N.GW_SIGNATURES, n
    assert set(N.GW_SIGNATURES) == set(names)


def test_every_workload_symbol_is_exported():
    names = _declared("gw_workload.h", "gww_")
    lib = N.libgw_workload()
    for n in names:
        assert hasattr(lib, n), n


def _engine(n=4, p=3, b=2):
    e = Engine(n, p, b, k_max=1)
    e.set_event_indices(np.zeros(n, dtype=np.int32))
    return e


MONO = [-1.0, 1.0, 0.9, 1.0, 1.2]


def test_bad_indices_rejected_at_add():
    e = _engine()
    with pytest.raises(N.GwError) as ex:
        e.add_spline(N.GW_DIAL_MONOTONIC, 0, 7, MONO)
    assert ex.value.code == N.GW_ERR_ARG and "Parameter index" in str(ex.value)
    with pytest.raises(N.GwError):
        e.add_spline(N.GW_DIAL_MONOTONIC, 9, 0, MONO)
    with pytest.raises(N.GwError):
        e.set_event_index(0, 5)
    with pytest.raises(N.GwError):
        e.add_spline(N.GW_DIAL_GRAPH, 0, 0, [1.0, 0.0])  # graph is not a spline type


@pytest.mark.parametrize("dial_type,data", [
    (N.GW_DIAL_MONOTONIC, [-1.0, 1.0, 0.9]),                      # one knot
    (N.GW_DIAL_MONOTONIC, [-1.0, 0.0, 0.9, 1.0]),                 # zero step
    (N.GW_DIAL_UNIFORM, [-1.0, 1.0, 0.9, 0.1, 1.0]),              # odd (y, dy) list
    (N.GW_DIAL_GENERAL, [0.0, 1.0, 1.0, 0.0, 0.5, 1.0, 0.0, 0.2]),  # x not increasing
])
def test_invalid_spline_data_rejected_before_device(dial_type, data):
    e = _engine()
    e.add_spline(dial_type, 0, 0, data)
    with pytest.raises(N.GwError) as ex:
        e.initialize()
    assert ex.value.code == N.GW_ERR_ARG and "invalid data" in str(ex.value)


def test_invalid_surface_and_tables_rejected():
    e = _engine()
    e.add_surface(N.GW_DIAL_BILINEAR, 0, 0, 1, [2.0, 2.0, 0.0, 1.0, 0.0, 1.0, 1.0, 1.0, 1.0])  # 3 of 4 knots
    with pytest.raises(N.GwError):
        e.initialize()
    e = _engine()
    t = e.create_table(10)
    e.add_kriged(0, t, [3, 12], [0.5, 0.5])  # index 12 outside a 10-entry table
    with pytest.raises(N.GwError):
        e.initialize()
    e = _engine()
    t = e.create_table(4)
    with pytest.raises(N.GwError) as ex:
        e.set_table(t, [1.0, np.nan, 1.0, 1.0])
    assert ex.value.code == N.GW_ERR_NOT_FINITE


def test_missing_bin_and_clamp_order_rejected():
    e = Engine(2, 1, 1, k_max=1)
    e.set_event_index(0, 0)
    with pytest.raises(N.GwError) as ex:
        e.initialize()
    assert ex.value.code == N.GW_ERR_STATE
    e = _engine()
    e.set_lower_clamp(1, 2.0)
    e.set_upper_clamp(1, 1.0)
    with pytest.raises(N.GwError) as ex:
        e.initialize()
    assert "clamp" in str(ex.value)


def test_event_larger_than_a_tile_is_a_limit_error():
    e = _engine(n=1, p=1, b=1)
    for _ in range(1100):
        e.reserve_norm(0, 0)
    with pytest.raises(N.GwError) as ex:
        e.initialize()
    assert ex.value.code == N.GW_ERR_LIMIT


def test_eval_before_initialize_is_a_state_error():
    e = _engine()
    with pytest.raises(N.GwError) as ex:
        e.eval(np.zeros((1, 3)))
    assert ex.value.code == N.GW_ERR_STATE


def test_bad_config_rejected():
    lib = N.libgw()
    cfg = N.GwConfig(10, 0, 1, 1, 0, 0, 0, 0)
    p = C.c_void_p()
    assert lib.gw_create(C.byref(cfg), C.byref(p)) == N.GW_ERR_ARG
    assert "bad gw_config" in N.last_error(None)
    cfg = N.GwConfig(10, 2, 1, 1, 0, 0, 0, 5)  # no such spline form
    assert lib.gw_create(C.byref(cfg), C.byref(p)) == N.GW_ERR_ARG
    cfg = N.GwConfig(10, 2, 1, 1, 3, 0, 0, 0)  # no such precision
    assert lib.gw_create(C.byref(cfg), C.byref(p)) == N.GW_ERR_ARG
    for flags in (0, N.GW_FLAG_SPLINE_KNOTS, N.GW_FLAG_SPLINE_SLOPES, N.GW_FLAG_SPLINE_COEFS,
                  N.GW_FLAG_SPLINE_GRID):
        for prec in (N.GW_FP64, N.GW_FP32, N.GW_DF64):
            cfg = N.GwConfig(10, 2, 1, 1, prec, 0, 0, flags)
            assert lib.gw_create(C.byref(cfg), C.byref(p)) == N.GW_OK
            lib.gw_destroy(p)


def test_eigen_block_validation():
    """gw_add_eigen_block refuses blocks outside the parameters, overlapping
    blocks and non-finite matrices (before any device work)."""
    import ctypes as C
    import numpy as np
    from gundam_gb300 import _native as N
    lib = N.libgw()
    cfg = N.GwConfig(10, 6, 4, 1, N.GW_FP64, 0, 0, 0)
    e = C.c_void_p()
    assert lib.gw_create(C.byref(cfg), C.byref(e)) == N.GW_OK
    V = np.eye(3)
    p = V.ctypes.data_as(C.c_void_p)
    assert lib.gw_add_eigen_block(e, 4, 3, p) == N.GW_ERR_ARG      # [4, 7) beyond 6 parameters
    assert lib.gw_add_eigen_block(e, 0, 3, p) == N.GW_OK
    assert lib.gw_add_eigen_block(e, 2, 3, p) == N.GW_ERR_ARG      # overlaps [0, 3)
    bad = np.eye(3)
    bad[1, 1] = np.nan
    assert lib.gw_add_eigen_block(e, 3, 3, bad.ctypes.data_as(C.c_void_p)) == N.GW_ERR_NOT_FINITE
    assert lib.gw_add_eigen_block(e, 3, 3, p) == N.GW_OK
    lib.gw_destroy(e)


def test_compiled_shape_list():
    """gw_shape_count / gw_shape_at list every compiled batched kernel shape
    (no device needed); out-of-range entries and selection before
    gw_initialize are argument / state errors."""
    shapes = Engine.compiled_shapes()
    assert len(shapes) >= 10
    for kind, ppp, ppt, threads, stages, minb in shapes:
        assert kind in (0, 1, 3) and threads in (128, 256) and stages in (1, 2) and minb >= 0
        if kind == 3:  # small-K warp-specialised: every evaluator thread takes all points of a pass
            assert ppp == ppt and ppp % 2 == 0 and threads == 256
        if kind == 0:
            assert ppp % ppt == 0 and ppp // ppt in (8, 16, 32)
    assert len(set(shapes)) == len(shapes)
    v = [C.c_int32() for _ in range(6)]
    lib = N.libgw()
    assert lib.gw_shape_at(len(shapes), *[C.byref(x) for x in v]) == N.GW_ERR_ARG
    assert lib.gw_shape_at(-1, *[C.byref(x) for x in v]) == N.GW_ERR_ARG
    e = _engine()
    with pytest.raises(N.GwError):
        e.set_shape_index(0)
    e.close()
