"""Golden bin sums from GUNDAM's own Cache::Manager calculators.

    python tests/golden/make_golden_cache.py

Needs oracle/_ref/libref_cache.so (python oracle/ref/build_ref.py <GUNDAM
tree>): the reference's Cache::Parameters / Cache::Weights / Cache::Weight::*
/ Cache::RecursiveSums compiled for the host and filled through its own
operator API (oracle/ref/ref_cache.cpp).  Writes tests/golden/cache_sums.npz:
for each case, the parameter points and the reference's per-bin sums of
weights and of squared weights.  Cases: the C1 workload (100k events, 3
points) and a 20k-event slice of C2 (every spline/graph/surface/norm type
of C2, 2 points).
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from gundam_gb300.workload import Workload  # noqa: E402
from oracle.oracle import RefCache  # noqa: E402

CASES = {"c1": ("c1", 0, 3, 31), "c2s": ("c2", 20000, 2, 32)}


def main():
    out = {}
    for name, (cfg, events, k, seed) in CASES.items():
        wl = Workload(cfg, n_events=events, seed=2)
        rc = RefCache(wl)
        pts = wl.draw_points(k, seed)
        s = np.empty((k, wl.n_bins))
        s2 = np.empty((k, wl.n_bins))
        for i in range(k):
            s[i], s2[i] = rc.eval(pts[i])
        rc.close()
        out[f"{name}_points"] = pts
        out[f"{name}_sums"] = s
        out[f"{name}_sums2"] = s2
        print(name, wl.n_events, wl.n_dials, s.sum())
    np.savez_compressed(Path(__file__).resolve().parent / "cache_sums.npz", **out)


if __name__ == "__main__":
    main()
