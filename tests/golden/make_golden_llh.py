"""Writes tests/golden/llh.json: per-bin likelihood values computed by the
reference's own classes (PoissonLogLikelihood.h:19-53 and
BarlowBeestonBanff2022.h:92-294, through oracle/_ref/libref_llh.so, built by
oracle/ref/build_ref.py from the GUNDAM source tree).  Each bin goes through
the reference's eval(SamplePair, bin) on a histogram holding (sum of
weights, sqrt of the sum of squared weights), as in a fit.

Run from the repository root:  python tests/golden/make_golden_llh.py
The cases: predictions <= 0 (both sides of the expected-value minimum),
empty data and data below the double epsilon, a zero sum of squared weights,
predictions down to 1e-300 (the fractional-error limit and the DBL_MIN
floor of the adjusted prediction), non-finite sums of squared weights, bins
where the default configuration throws (a non-finite chi2, a negative root),
and random bins over nine decades of prediction and weight.
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle.oracle import ref_llh_bins  # noqa: E402

POISSON, BB = 1, 2


def cases():
    rng = np.random.default_rng(20261204)
    rows = []
    preds = [-2.0, -1.0, -0.5, 0.0, 1e-300, 1e-200, 1e-160, 1e-154, 1e-100, 1e-20, 1e-16, 1e-8, 1e-3, 0.5, 1.0,
             3.0, 17.25, 1e3, 1e6]
    datas = [0.0, 1e-17, 2.220446049250313e-16, 1e-15, 1.0, 2.0, 7.0, 1e3]
    sqrts = [0.0, 1e-3, 0.5, 1.0, 3.0, 1e2]
    for p in preds:
        for d in datas:
            for s in sqrts:
                rows.append((d, p, s))
    for s in (float("inf"), float("nan")):
        rows.append((2.0, 5.0, s))
    # bins whose chi2 is not finite or whose root is negative: the default
    # configuration throws there
    rows += [(1e10, 1e-300, 1e2), (1e200, 1e-300, 1e2), (-5.0, 1.0, 10.0), (-1e3, 0.5, 3.0)]
    # random bins: prediction log-uniform over nine decades, data a Poisson
    # draw of it, sum of squared weights = prediction x mean weight
    p = 10.0 ** rng.uniform(-4, 5, 600)
    d = rng.poisson(p).astype(np.float64)
    wbar = 10.0 ** rng.uniform(-3, 1, 600)
    for a, b, c in zip(d, p, np.sqrt(p * wbar)):
        rows.append((float(a), float(b), float(c)))
    return rows


def enc(x):
    return x if np.isfinite(x) else ("inf" if x > 0 else ("-inf" if x < 0 else "nan"))


def main():
    rows = cases()
    data = np.array([r[0] for r in rows])
    pred = np.array([r[1] for r in rows])
    sq = np.array([r[2] for r in rows])
    out = {"source": "reference PoissonLogLikelihood / BarlowBeestonBanff2022 via eval(SamplePair, bin)",
           "columns": ["data", "pred", "sqrt_sum_w2", "poisson", "bb", "bb_default_throws"],
           "bb_default_throws": "0 returns, 1 throws (the engine returns +inf), 2 ends the process", "rows": []}
    r_p = ref_llh_bins(POISSON, data, pred, sq)
    r_b = ref_llh_bins(BB, data, pred, sq)
    if r_p is None or r_b is None:
        raise SystemExit("oracle/_ref/libref_llh.so is missing; build it first")
    for i in range(len(rows)):
        out["rows"].append([enc(data[i]), enc(pred[i]), enc(sq[i]), enc(r_p[0][i]), enc(r_b[0][i]),
                            int(r_b[1][i])])
    path = ROOT / "tests" / "golden" / "llh.json"
    head = {k: v for k, v in out.items() if k != "rows"}
    text = json.dumps(head)[:-1] + ', "rows": [\n' + ",\n".join(json.dumps(r) for r in out["rows"]) + "\n]}\n"
    path.write_text(text)
    print(f"{len(rows)} bins -> {path}")


if __name__ == "__main__":
    main()
