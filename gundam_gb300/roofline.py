"""Algorithmic bytes of one evaluation pass (the roofline numerator).

One pass reads every dial's payload, its index data and the per-event data
once, whatever the number K of parameter points it serves, and moves K
parameter vectors in and K bin vectors (sum of w, sum of w^2, FP64) out:

  bytes(K) = sum_dials payload(type, s) + D*6 + N*(4 + s + 4) + tables
             + K*(P*8 + B*16)

with s = 8 (FP64) or 4 (FP32) bytes per stored value and
  payload = s*(2+n) monotonic/compact, s*(2+2n) uniform, s*(2+3n) general,
            s*2n graph, s*(2+nx+ny+nx*ny) surfaces, 0 norm,
            (4+s) tabulated, 8m kriged.
"""
from __future__ import annotations

import numpy as np

from . import _native as N


def algorithmic_bytes(wl, precision: str, K: int) -> int:
    s = 4 if precision == "fp32" else 8
    t = wl.dial_type.astype(np.int64)
    lens = np.diff(wl.dial_data_start)
    values = (t != N.GW_DIAL_TABULATED) & (t != N.GW_DIAL_KRIGED)
    payload = int(lens[values].sum()) * s
    payload += int((t == N.GW_DIAL_TABULATED).sum()) * (4 + s)
    kr = t == N.GW_DIAL_KRIGED
    if kr.any():
        m = (lens[kr] - 2) // 2
        payload += int(m.sum()) * 8
    tables = int(wl.table_size.sum()) * s if wl.n_tables else 0
    D, Nev, P, B = wl.n_dials, wl.n_events, wl.n_params, wl.n_bins
    return payload + D * 6 + Nev * (4 + s + 4) + tables + K * (P * 8 + B * 16)


# FP32 operations per dial and point, counted on the restated formulas
# (Hermite spline: index, fraction, cubic; graph: search + linear; bilinear:
# three linear interpolations), plus one multiply per dial for the event
# product and, per event and point, the cap, the base weight and the FP64
# w and w^2 accumulations (counted as 4).
FLOPS_PER_DIAL = {
    N.GW_DIAL_NORM: 1, N.GW_DIAL_MONOTONIC: 30, N.GW_DIAL_UNIFORM: 20, N.GW_DIAL_GENERAL: 35,
    N.GW_DIAL_COMPACT: 30, N.GW_DIAL_GRAPH: 12, N.GW_DIAL_BILINEAR: 20, N.GW_DIAL_BICUBIC: 60,
    N.GW_DIAL_TABULATED: 3,
}


def algorithmic_flops(wl, K: int) -> int:
    """FP32-equivalent operations of one pass over all events for K points."""
    t = wl.dial_type.astype(np.int64)
    counts = np.bincount(t, minlength=16)
    per_point = 0
    for typ, f in FLOPS_PER_DIAL.items():
        per_point += int(counts[typ]) * (f + 1)
    kr = t == N.GW_DIAL_KRIGED
    if kr.any():
        lens = np.diff(wl.dial_data_start)[kr]
        per_point += int(((lens - 2) // 2).sum()) * 2 + int(kr.sum())
    per_point += wl.n_events * 4
    return per_point * K
