"""The oracle against the reference's own dial functions.

tests/golden/dials.json holds responses computed by the reference's
src/Utils/include/Calculate*.h (made by tests/golden/make_golden.py through
oracle/_ref).  The oracle must reproduce them bit for bit.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = json.loads((Path(__file__).parent / "golden" / "dials.json").read_text())


def test_golden_fixture_covers_every_function_type():
    types = {c[0] for c in GOLDEN["cases"]}
    assert types == {2, 3, 4, 5, 6, 7, 8}
    assert len(GOLDEN["cases"]) > 3000


def test_oracle_matches_reference_golden_bit_exact():
    data = GOLDEN["data"]
    mism = []
    for t, di, x, y, v in GOLDEN["cases"]:
        got = O.dial(t, data[di], x, y, False)
        if not (got == v or (np.isnan(got) and np.isnan(v))):
            mism.append((t, di, x, y, v, got))
    assert not mism, f"{len(mism)} mismatches, first: {mism[:3]}"


@pytest.mark.skipif(O.ref_lib() is None, reason="oracle/_ref not built (reference tree absent)")
def test_oracle_matches_reference_on_fresh_random_knots():
    ref = O.ref_lib()
    rng = np.random.default_rng(99)
    for trial in range(300):
        n = int(rng.integers(2, 20))
        lo, step = float(rng.uniform(-3, 0)), float(rng.uniform(0.1, 1.0))
        ys = np.exp(rng.normal(0, 0.4, n))
        d = np.array([lo, step, *ys])
        for x in rng.uniform(lo - 3, lo + (n - 1) * step + 3, 20):
            r = ref.ref_monotonic(float(x), -1e20, 1e20, d.ctypes.data, len(d))
            assert O.dial(2, d, float(x)) == r
            r = ref.ref_compact(float(x), -1e20, 1e20, d.ctypes.data, len(d))
            assert O.dial(5, d, float(x)) == r
        xk = np.sort(np.concatenate([[lo, lo + 5], rng.uniform(lo + 0.01, lo + 4.99, max(0, n - 2))]))
        g = np.array([v for pair in zip(ys, xk) for v in pair])
        gd = np.array([xk[0], 1.0, *[v for t in zip(ys, rng.normal(0, 1, n), xk) for v in t]])
        for x in rng.uniform(lo - 3, lo + 8, 20):
            assert O.dial(6, g, float(x)) == ref.ref_graph(float(x), -1e20, 1e20, g.ctypes.data, len(g))
            assert O.dial(4, gd, float(x)) == ref.ref_general(float(x), -1e20, 1e20, gd.ctypes.data, len(gd))
