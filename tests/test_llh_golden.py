"""The per-bin likelihood against the reference's own classes.

tests/golden/llh.json holds per-bin values computed by GUNDAM's
PoissonLogLikelihood (PoissonLogLikelihood.h:19-53) and
BarlowBeestonBanff2022 (BarlowBeestonBanff2022.h:92-294) through their
eval(SamplePair, bin), made by tests/golden/make_golden_llh.py through
oracle/_ref.  The oracle must reproduce them bit for bit; the engine's device
terms are checked against the same fixture in tests/test_gpu_llh.py.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = json.loads((Path(__file__).parent / "golden" / "llh.json").read_text())


def _f(x):
    return float(x)  # "inf", "nan" and numbers alike


def rows():
    r = GOLDEN["rows"]
    return (np.array([_f(x[0]) for x in r]), np.array([_f(x[1]) for x in r]), np.array([_f(x[2]) for x in r]),
            np.array([_f(x[3]) for x in r]), np.array([_f(x[4]) for x in r]), np.array([x[5] for x in r]))


def _same(a, b):
    return (a == b) | (np.isnan(a) & np.isnan(b))


def test_fixture_covers_the_edge_cases():
    data, pred, sq, po, bb, th = rows()
    assert len(data) > 1500
    assert np.any(pred <= -1.0) and np.any((pred <= 0) & (pred > -1.0))  # both sides of the minimum
    assert np.any(data == 0.0) and np.any((data > 0) & (data <= np.finfo(float).eps))
    assert np.any(sq == 0.0) and np.any(~np.isfinite(sq))
    assert np.any(pred <= 1e-154) and np.any(np.isinf(po)) and np.any(np.isinf(bb))
    assert np.any(th == 1) and np.any(th == 2)


@pytest.mark.parametrize("llh_type", [1, 2])
def test_oracle_matches_reference_likelihood_bit_exact(llh_type):
    data, pred, sq, po, bb, _ = rows()
    ref = po if llh_type == 1 else bb
    got = np.array([O.llh_bin(llh_type, d, p, s) for d, p, s in zip(data, pred, sq)])
    bad = ~_same(got, ref)
    assert not bad.any(), f"{bad.sum()} mismatches, first: {list(zip(data[bad], pred[bad], sq[bad], got[bad]))[:3]}"


@pytest.mark.skipif(O.ref_llh_lib() is None, reason="oracle/_ref not built (reference tree absent)")
@pytest.mark.parametrize("llh_type", [1, 2])
def test_oracle_matches_reference_likelihood_on_fresh_bins(llh_type):
    rng = np.random.default_rng(123)
    pred = 10.0 ** rng.uniform(-6, 6, 4000)
    data = rng.poisson(np.minimum(pred, 1e9)).astype(np.float64)
    sq = np.sqrt(pred * 10.0 ** rng.uniform(-4, 2, 4000))
    ref, _ = O.ref_llh_bins(llh_type, data, pred, sq)
    got = np.array([O.llh_bin(llh_type, d, p, s) for d, p, s in zip(data, pred, sq)])
    assert _same(got, ref).all()
