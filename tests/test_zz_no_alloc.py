"""gw_llh_noalloc: the likelihood for callers that cannot allocate device memory.

Such callers (code inside a framework that owns the GPU's memory, or
per-evaluation callbacks that must not let cudaMalloc/cudaFree synchronise the
device) pass bin sums they already hold on the device; the library keeps the
reduction's scratch in a fixed array of its own.  The result must match the
likelihood gw_eval computes from the same sums, on two calls in a row (the
scratch keeps the previous call's contents).  This file runs last.
"""
import ctypes as C

import numpy as np
import pytest

from gundam_gb300 import Engine, Workload
from gundam_gb300 import _native as N

pytestmark = pytest.mark.gpu

LLH_ABS = 1e-6  # the FP64 likelihood tolerance of the parity tests


def _vp(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("config,llh_type", [("c1", N.GW_LLH_POISSON), ("mixed", N.GW_LLH_BARLOW_BEESTON_OA2021)])
def test_noalloc_llh_matches_engine_twice(config, llh_type):
    torch = pytest.importorskip("torch")
    wl = Workload(config, seed=13)
    K = 16
    eng = Engine.from_workload(wl, precision="fp64", k_max=K, llh_type=llh_type)
    pts = wl.draw_points(K, 3)
    d_p = torch.from_numpy(pts).cuda()
    d_s = torch.empty((K, wl.n_bins), dtype=torch.float64, device="cuda")
    d_s2 = torch.empty_like(d_s)
    d_stat = torch.empty(K, dtype=torch.float64, device="cuda")
    d_data = torch.from_numpy(np.ascontiguousarray(wl.data)).cuda()
    stream = torch.cuda.Stream()
    eng.eval_device(d_p.data_ptr(), K, d_s.data_ptr(), d_s2.data_ptr(), 0, d_stat.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    eng.sync()
    ref = d_stat.cpu().numpy()
    lib = N.libgw()
    for call in range(2):
        out = torch.full((K,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.gw_llh_noalloc(_vp(d_s), _vp(d_s2), _vp(d_data), wl.n_bins, K, llh_type, _vp(out),
                                C.c_void_p(stream.cuda_stream))
        assert rc == N.GW_OK, N.last_error(None)
        stream.synchronize()
        got = out.cpu().numpy()
        fin = np.isfinite(ref)
        assert np.array_equal(np.isfinite(got), fin), f"call {call}"
        assert np.max(np.abs(got[fin] - ref[fin]), initial=0.0) <= LLH_ABS, f"call {call}"
    eng.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = N.libgw()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    # 4097 points exceed the 4096 counters
    rc = lib.gw_llh_noalloc(_vp(d), _vp(d), _vp(d), 1, 4097, N.GW_LLH_POISSON, _vp(d), None)
    assert rc == N.GW_ERR_LIMIT
    assert "65536" in N.last_error(None)
    # 300 points x 256 blocks of bins exceed the 65536 block partials
    rc = lib.gw_llh_noalloc(_vp(d), _vp(d), _vp(d), 256 * 256, 300, N.GW_LLH_POISSON, _vp(d), None)
    assert rc == N.GW_ERR_LIMIT


def test_noalloc_request_exactly_at_the_bound():
    """K * ceil(n_bins / 256) == 65536 exactly (256 points of 65536 bins): the
    last block partial lands at the end of the array, next to the counters.
    Accepted, and equal to a host sum of the same per-bin Poisson terms, on
    two calls in a row."""
    torch = pytest.importorskip("torch")
    import math

    K, B = 256, 65536
    rng = np.random.default_rng(17)
    sums = rng.uniform(0.5, 40.0, size=(K, B))
    data = rng.poisson(sums[0]).astype(np.float64)
    ref = []
    for k in range(K):
        p = sums[k]
        term = np.where(data <= 0.0, 2.0 * p, 2.0 * (p - data + data * np.log(np.where(data > 0, data, 1.0) / p)))
        ref.append(math.fsum(term.tolist()))
    ref = np.array(ref)
    d_s = torch.from_numpy(sums).cuda()
    d_s2 = torch.from_numpy(sums * 0.01).cuda()
    d_data = torch.from_numpy(data).cuda()
    lib = N.libgw()
    for call in range(2):
        out = torch.full((K,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.gw_llh_noalloc(_vp(d_s), _vp(d_s2), _vp(d_data), B, K, N.GW_LLH_POISSON, _vp(out), None)
        assert rc == N.GW_OK, N.last_error(None)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got)), f"call {call}"
        assert np.max(np.abs(got - ref)) <= LLH_ABS, f"call {call}"
