"""The engine's per-bin likelihood terms (the device functions gw_eval sums)
against values computed by the reference's own classes (tests/golden/llh.json,
see tests/test_llh_golden.py), through the C ABI (gw_llh_bins).

Tolerance: 1e-13 of the bin's scale |term| + |data| + |pred| (device and
host logarithms may differ in the last bit, and where data and prediction
nearly agree the term is a small difference of large ones, so the bound is on
the error relative to the operands, as for any cancelling sum); non-finite
reference values must be matched exactly (+inf, NaN)."""
import numpy as np
import pytest

from gundam_gb300 import _native as N
from tests.test_llh_golden import rows

pytestmark = pytest.mark.gpu

REL = 1e-13


@pytest.mark.parametrize("llh_type", [N.GW_LLH_POISSON, N.GW_LLH_BARLOW_BEESTON_OA2021])
def test_device_terms_match_reference_classes(llh_type):
    data, pred, sq, po, bb, _ = rows()
    ref = po if llh_type == N.GW_LLH_POISSON else bb
    out = np.full(data.size, -1.0)
    rc = N.libgw().gw_llh_bins(llh_type, data.ctypes.data, pred.ctypes.data, sq.ctypes.data, data.size,
                               out.ctypes.data)
    assert rc == N.GW_OK
    fin = np.isfinite(ref)
    assert np.array_equal(np.isposinf(out), np.isposinf(ref))
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    den = np.maximum(np.abs(ref[fin]) + np.abs(data[fin]) + np.abs(pred[fin]), 1e-300)
    err = np.abs(out[fin] - ref[fin]) / den
    assert err.max(initial=0.0) <= REL, (err.max(), data[fin][err.argmax()], pred[fin][err.argmax()])
