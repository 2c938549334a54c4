"""Writes tests/golden/dials.json: dial responses computed by the reference's
own src/Utils/include/Calculate*.h (through oracle/_ref/libref_dials.so,
built by oracle/ref/build_ref.py from the GUNDAM source tree).

Run from the repository root:  python tests/golden/make_golden.py
The cases cover every knot-count edge the reference's unit tests use
(tests/GTests/unitTest_Calculate*.cpp) plus random knot sets, with x inside,
on the knots, on the ends and far outside (extrapolation).
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle.oracle import ref_lib  # noqa: E402

MONOTONIC, UNIFORM, GENERAL, COMPACT, GRAPH, BILINEAR, BICUBIC = 2, 3, 4, 5, 6, 7, 8


def xs_for(lo, hi, knots, rng, n=24):
    xs = list(np.linspace(lo - 2.0, hi + 2.0, 9)) + list(knots) + [lo, hi, lo - 7.5, hi + 7.5]
    xs += list(rng.uniform(lo - 1.0, hi + 1.0, n))
    return [float(x) for x in xs]


def main():
    ref = ref_lib()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_dials.so is missing; build it first")
    rng = np.random.default_rng(20261203)
    cases = []

    def call1(fn, x, d):
        a = np.ascontiguousarray(d, dtype=np.float64)
        return getattr(ref, fn)(x, -1e20, 1e20, a.ctypes.data, len(a))

    def call2(fn, x, y, d):
        a = np.ascontiguousarray(d, dtype=np.float64)
        return getattr(ref, fn)(x, y, -1e20, 1e20, a.ctypes.data, len(a))

    # fixed knot sets from the reference's unit tests (monotonic 2/3/6/13/17 knots,
    # the 7-point DialDefinitions fixture) and random ones
    fixed = [
        [0.0, 1.0],
        [0.0, 1.0, 0.0],
        [0.0, 0.0, 1.0, 1.0, 0.0, 0.0],
        [0.5, 1.5, 1.0, 1.0, 1.0, 1.0, 0.5, 1.0, 1.0, 1.0, 1.0, 1.5, 0.5],
        [float(np.cos(4.0 * (-1 + 2 * i / 16))) for i in range(17)],
        [1.75, 1.5, 1.0, 0.0, 1.0, 1.5, 1.75],
    ]
    for ys in fixed + [list(np.cumsum(rng.uniform(0.0, 0.5, n)) * rng.choice([-1, 1]) + 1.0)
                       for n in (2, 3, 4, 5, 7, 9, 12, 16, 20, 31)]:
        n = len(ys)
        lo = -1.0 if n != 7 else -3.0
        step = (2.0 if n != 7 else 6.0) / max(1, n - 1)
        knots = [lo + i * step for i in range(n)]
        d = [lo, step] + list(ys)
        for t, fn in ((MONOTONIC, "ref_monotonic"), (COMPACT, "ref_compact")):
            for x in xs_for(knots[0], knots[-1], knots, rng):
                cases.append({"type": t, "data": d, "x": x, "y": 0.0, "v": call1(fn, x, d)})
    # uniform splines with Catmull-Rom slopes
    for n in (2, 3, 5, 7, 11, 16, 31):
        lo, hi = -3.0, 3.0
        step = (hi - lo) / (n - 1)
        xk = np.array([lo + i * step for i in range(n)])
        yk = np.exp(rng.normal(0, 0.3, n))
        dy = np.gradient(yk, xk) if n > 2 else np.full(n, (yk[-1] - yk[0]) / (xk[-1] - xk[0]))
        d = [lo, step] + [float(v) for pair in zip(yk, dy) for v in pair]
        for x in xs_for(lo, hi, xk, rng):
            cases.append({"type": UNIFORM, "data": d, "x": x, "y": 0.0, "v": call1("ref_uniform", x, d)})
    # general splines, non-uniform knots
    for n in (2, 3, 5, 8, 15, 17, 31):
        xk = np.sort(np.concatenate([[-3.0, 3.0], rng.uniform(-2.9, 2.9, n - 2)]))
        yk = np.exp(rng.normal(0, 0.3, n))
        dy = rng.normal(0, 0.5, n)
        d = [float(xk[0]), float((xk[-1] - xk[0]) / (n - 1))] + [float(v) for t in zip(yk, dy, xk) for v in t]
        for x in xs_for(xk[0], xk[-1], xk, rng):
            cases.append({"type": GENERAL, "data": d, "x": x, "y": 0.0, "v": call1("ref_general", x, d)})
    # graphs (1..31 points)
    for n in (1, 2, 3, 4, 7, 15, 16, 31):
        xk = np.sort(np.concatenate([[-3.0, 3.0], rng.uniform(-2.9, 2.9, max(0, n - 2))]))[:n]
        if n == 1:
            xk = np.array([0.25])
        yk = np.exp(rng.normal(0, 0.3, n))
        d = [float(v) for t in zip(yk, xk) for v in t]
        for x in xs_for(float(xk[0]), float(xk[-1]), xk, rng):
            cases.append({"type": GRAPH, "data": d, "x": x, "y": 0.0, "v": call1("ref_graph", x, d)})
    # surfaces
    for nx, ny in ((2, 2), (3, 4), (5, 5), (7, 3), (16, 16), (17, 5)):
        xx = np.sort(np.concatenate([[-3.0, 3.0], rng.uniform(-2.9, 2.9, nx - 2)]))
        yy = np.sort(np.concatenate([[-2.0, 2.5], rng.uniform(-1.9, 2.4, ny - 2)]))
        z = np.exp(rng.normal(0, 0.3, nx * ny))
        d = [float(nx), float(ny)] + [float(v) for v in xx] + [float(v) for v in yy] + [float(v) for v in z]
        pts = [(float(a), float(b)) for a, b in zip(rng.uniform(-5, 5, 40), rng.uniform(-4, 4.5, 40))]
        pts += [(float(a), float(b)) for a in xx[:3] for b in yy[:3]]
        pts += [(-3.0, -2.0), (3.0, 2.5), (-9.0, 7.0), (9.0, -7.0)]
        for x, y in pts:
            cases.append({"type": BILINEAR, "data": d, "x": x, "y": y, "v": call2("ref_bilinear", x, y, d)})
            if nx >= 2 and ny >= 2:
                cases.append({"type": BICUBIC, "data": d, "x": x, "y": y, "v": call2("ref_bicubic", x, y, d)})
    # store every data vector once; a case is [type, data index, x, y, value]
    datasets, index, rows = [], {}, []
    for c in cases:
        key = tuple(c["data"])
        if key not in index:
            index[key] = len(datasets)
            datasets.append(c["data"])
        rows.append([c["type"], index[key], c["x"], c["y"], c["v"]])
    out = Path(__file__).resolve().parent / "dials.json"
    with open(out, "w") as f:
        json.dump({"source": "src/Utils/include/Calculate*.h via oracle/_ref",
                   "columns": ["type", "data", "x", "y", "value"], "data": datasets, "cases": rows}, f,
                  separators=(",", ":"))
    print(f"wrote {len(rows)} cases over {len(datasets)} data vectors to {out}")


if __name__ == "__main__":
    main()
