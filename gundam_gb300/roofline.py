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
