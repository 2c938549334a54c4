"""The oracle against GUNDAM's own Cache::Manager calculators.

tests/golden/cache_sums.npz holds per-bin sums of weights and of squared
weights computed by the reference's Cache::Parameters / Cache::Weights /
Cache::Weight::* / Cache::RecursiveSums, compiled for the host from the
reference tree and filled through its own operator API
(tests/golden/make_golden_cache.py, oracle/ref/ref_cache.cpp).  The oracle
restates the CPU propagation; on these workloads (no clamped norms, no weight
cap, extrapolation allowed) the two paths agree on every occupied bin to
rounding (the reference reduces bins pairwise and multiplies the dials
calculator by calculator, the oracle in event order).  Empty bins are the one
documented difference: RecursiveSums hands an empty bin the content of the
next bin (CacheRecursiveSums.cpp:271-279), the CPU path gives 0.
"""
from pathlib import Path

import numpy as np
import pytest

from gundam_gb300 import _native as N
from gundam_gb300.workload import Workload

GOLD = Path(__file__).resolve().parent / "golden" / "cache_sums.npz"
CASES = {"c1": ("c1", 0), "c2s": ("c2", 20000)}


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_cache_manager_fixtures(name):
    from oracle.oracle import Oracle
    cfg, events = CASES[name]
    g = np.load(GOLD)
    wl = Workload(cfg, n_events=events, seed=2)
    o = Oracle(wl, N.GW_LLH_POISSON)
    r = o.eval(g[f"{name}_points"])
    occupied = np.bincount(wl.event_bin, minlength=wl.n_bins) > 0
    for key, ref in (("sums", g[f"{name}_sums"]), ("sums2", g[f"{name}_sums2"])):
        rel = np.abs(r[key] - ref)[:, occupied] / np.abs(ref[:, occupied])
        assert rel.max() < 1e-12, (name, key, rel.max())
        assert np.all(r[key][:, ~occupied] == 0.0)
    o.close()


def test_oracle_matches_live_reference_cache_manager():
    from oracle.oracle import Oracle, RefCache, ref_cache_lib
    if ref_cache_lib() is None:
        pytest.skip("oracle/_ref/libref_cache.so not built here")
    wl = Workload("c2", n_events=5000, seed=7)
    rc = RefCache(wl)
    o = Oracle(wl, N.GW_LLH_POISSON)
    pts = wl.draw_points(2, 77)
    counts = np.bincount(wl.event_bin, minlength=wl.n_bins)
    occ = counts > 0
    for k in range(2):
        s, s2, w = rc.eval(pts[k], weights=True)
        r = o.eval(pts[k:k + 1], weights=True)
        np.testing.assert_allclose(s[occ], r["sums"][0][occ], rtol=1e-12, atol=0)
        np.testing.assert_allclose(s2[occ], r["sums2"][0][occ], rtol=1e-12, atol=0)
        np.testing.assert_allclose(w, r["weights"], rtol=1e-13, atol=1e-300)
        # the documented empty-bin difference: the reference copies the next
        # occupied bin's content, the CPU path (and the engine) gives 0
        empty = np.nonzero(~occ)[0]
        assert empty.size > 0
        for b in empty[:20]:
            nxt = b + 1 + int(np.argmax(occ[b + 1:])) if b + 1 < wl.n_bins and occ[b + 1:].any() else None
            assert r["sums"][0][b] == 0.0
            if nxt is not None:
                assert s[b] == s[nxt]
    rc.close()
    o.close()
