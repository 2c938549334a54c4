"""Engine features on the GPU: the Cache::Manager interface, the stress
configuration's device-side kriging table, and the bounded-wait failure path."""
import ctypes as C

import numpy as np
import pytest

from gundam_gb300 import CacheManager, Engine, Workload
from gundam_gb300 import _native as N
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    den = np.where(b != 0, np.abs(b), 1.0)
    return float(np.max(np.abs(a - b) / den))


def test_cache_manager_interface_matches_oracle():
    wl = Workload("c1", n_events=20000, seed=8)
    orc = Oracle(wl, llh_type=N.GW_LLH_POISSON)
    assert CacheManager.HasCUDA() and CacheManager.HasGPU()
    CacheManager.SetIsEnabled(True)
    old = CacheManager.SetIsEventWeightCopyEnabled(True)
    assert CacheManager.Build(wl, precision="fp64")
    p = wl.draw_points(1, 4)
    fut = CacheManager.Fill(p)
    assert fut.valid() and fut.get() and not fut.valid()
    cm = CacheManager.Get()
    ref = orc.eval(p, weights=True)
    sw, err = cm.CopyHistogramContents()
    assert _rel(sw, ref["sums"][0]) <= 1e-12
    assert cm.ValidateHistogramContents(ref["sums"][0], np.sqrt(ref["sums2"][0]))
    assert _rel(cm.weights, ref["weights"]) <= 1e-13
    assert abs(cm.llh - ref["llh"][0]) <= 1e-6
    assert cm.GetResidentMemory() > 0
    CacheManager.SetIsEventWeightCopyEnabled(old)
    CacheManager.Reset()
    assert not CacheManager.Fill(p).valid()


@pytest.mark.parametrize("precision,K,rel,ab", [("fp64", 1, 1e-12, 1e-6), ("fp64", 4, 1e-12, 1e-6),
                                              ("fp32", 8, 2e-5, 5e-2)])
def test_c5_slice_with_device_kriging_table(precision, K, rel, ab):
    wl = Workload("c5", n_events=150000, seed=9)
    assert wl.n_tables == 1 and wl.table_fn_par[0, 0] == 394
    orc = Oracle(wl, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021)
    eng = Engine.from_workload(wl, precision=precision, k_max=K)
    pts = wl.draw_points(K, 10)
    sums, sums2, llh, stat = eng.eval(pts)
    ref = orc.eval(pts)
    assert _rel(sums, ref["sums"]) <= rel
    assert _rel(sums2, ref["sums2"]) <= rel
    assert np.max(np.abs(llh - ref["llh"])) <= ab
    eng.close()


def test_bounded_wait_gives_up_and_reports():
    t = C.c_int32(-1)
    assert N.libgw().gw_selftest_wait_timeout(2000, C.byref(t)) == N.GW_OK
    assert t.value == 1
    # the context is still usable afterwards
    wl = Workload("mixed", seed=2)
    eng = Engine.from_workload(wl, precision="fp64", k_max=1, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021)
    s, s2, l, st = eng.eval(wl.nominal())
    assert np.isfinite(l[0])
    eng.close()
