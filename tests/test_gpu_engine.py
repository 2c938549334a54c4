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


@pytest.mark.parametrize("graph", [False, True])
def test_device_and_host_evaluations_on_two_streams_are_ordered(graph):
    """gw_eval_device on a caller stream followed at once, with no host
    synchronisation, by gw_eval on the engine's stream (and the reverse): both
    use the engine's one set of scratch arrays, so the engine must order them.
    Each result is checked against the oracle."""
    torch = pytest.importorskip("torch")
    wl = Workload("c1", seed=12)
    orc = Oracle(wl, llh_type=N.GW_LLH_POISSON)
    K = 8
    eng = Engine.from_workload(wl, precision="fp64", k_max=K, llh_type=N.GW_LLH_POISSON)
    eng.use_graph(graph)
    pa = wl.draw_points(K, 21)
    pb = wl.draw_points(K, 22)
    ref_a, ref_b = orc.eval(pa), orc.eval(pb)
    d_p = torch.from_numpy(pa).cuda()
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    for rep in range(3):
        d_s = torch.full((K, wl.n_bins), float("nan"), dtype=torch.float64, device="cuda")
        d_s2 = torch.full_like(d_s, float("nan"))
        d_l = torch.full((K,), float("nan"), dtype=torch.float64, device="cuda")
        d_st = torch.full_like(d_l, float("nan"))
        torch.cuda.synchronize()
        eng.eval_device(d_p.data_ptr(), K, d_s.data_ptr(), d_s2.data_ptr(), d_l.data_ptr(), d_st.data_ptr(),
                        stream.cuda_stream)
        sums, sums2, llh, stat = eng.eval(pb)  # engine stream, no host sync in between
        eng.eval_device(d_p.data_ptr(), K, d_s.data_ptr(), d_s2.data_ptr(), d_l.data_ptr(), d_st.data_ptr(),
                        stream.cuda_stream)
        stream.synchronize()
        eng.sync()
        assert _rel(sums, ref_b["sums"]) <= 1e-12, rep
        assert _rel(sums2, ref_b["sums2"]) <= 1e-12, rep
        assert np.max(np.abs(llh - ref_b["llh"])) <= 1e-6, rep
        assert _rel(d_s.cpu().numpy(), ref_a["sums"]) <= 1e-12, rep
        assert _rel(d_s2.cpu().numpy(), ref_a["sums2"]) <= 1e-12, rep
        assert np.max(np.abs(d_l.cpu().numpy() - ref_a["llh"])) <= 1e-6, rep
    eng.close()
