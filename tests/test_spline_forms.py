"""The engine's three evaluation forms of uniform-knot Catmull-Rom splines,
restated in numpy, against the oracle (which matches the reference's own
CalculateMonotonicSpline.h / CalculateCompactSpline.h bit for bit).

The engine stores a Catmull-Rom spline either as knot values, with the two
slopes of the interval formed on the device (`eval_knots`, gw_dials.cuh), or
with the knot slopes precomputed on the host (`write_prepared`,
gw_engine.cpp) and evaluated one point at a time (`eval_prepared`) or two
points at a time in packed FP32 with the cubic rearranged (`eval_prepared2`).
These checks pin the arithmetic of those forms on the CPU: the slope rule and
its end-knot cases, the interval and extrapolation rules, and the rearranged
Hermite cubic, in FP64 (to 1e-12 of the knot scale) and in FP32 arithmetic
(to 2e-5).  The same for the per-interval coefficient blocks that the
coefficient and grid forms store (Catmull-Rom and uniform splines, the
extrapolation blocks re-expanded about their own origin).  The GPU parity
tests run the compiled kernels.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

MONOTONIC, COMPACT = 2, 5


def host_slopes(y, limit):
    """write_prepared: knot slopes in index units (Fritsch-Carlson limited when `limit`)."""
    n = len(y)
    s = np.empty(n)
    for k in range(n):
        if k == 0:
            s[k] = y[1] - y[0]
        elif k == n - 1:
            s[k] = y[n - 1] - y[n - 2]
        else:
            s[k] = knot_slope(y[k] - y[k - 1], y[k + 1] - y[k], limit)
    return s


def knot_slope(dl, dr, limit):
    """knot_slope (gw_dials.cuh); the same operations for both stored forms."""
    s = 0.5 * (dl + dr)
    if limit:
        if dr * dl <= 0:
            s = 0.0 * s
        delta = 3 * min(abs(dl), abs(dr))
        if s > delta:
            s = delta
        if s < -delta:
            s = -delta
    return s


def interval(xx, n, trunc, f):
    """knot_interval: clamp to the knot range when truncating, i = clamp(floor(xx), 0, n - 2)."""
    if trunc:
        xx = min(max(xx, f(0)), f(n - 1))
    fi = min(max(f(math.floor(xx)), f(0)), f(n - 2))
    return xx, fi, int(fi)


def hermite(p1, m1, p2, m2, fx):
    return ((((2 * p1 - 2 * p2 + m2 + m1) * fx + 3 * p2 - 3 * p1 - m2 - 2 * m1) * fx + m1) * fx + p1)


def hermite_packed(p1, m1, p2, m2, fx):
    """eval_prepared2's form: p1 + fx(m1 + fx(B + fx A))."""
    dc = p2 - p1
    a = (-2 * dc + m2) + m1
    b = -2 * m1 + (3 * dc - m2)
    return ((a * fx + b) * fx + m1) * fx + p1


def evaluate(form, low, inv, y, s, x, trunc, catmull, f):
    xx = (f(x) - f(low)) * f(inv)
    xx, fi, i = interval(xx, len(y), trunc, f)
    fx = xx - fi
    p1, p2 = f(y[i]), f(y[i + 1])
    if form == "knots":
        dc = p2 - p1
        dl = p1 - f(y[i - 1]) if i > 0 else dc
        dr = f(y[i + 2]) - p2 if i + 2 < len(y) else dc
        m1, m2 = knot_slope(dl, dc, catmull), knot_slope(dc, dr, catmull)
    else:
        m1, m2 = f(s[i]), f(s[i + 1])
    if fx < 0:
        m2 = p2 - p1
    if fx >= 1:
        m1 = p2 - p1
    return (hermite_packed if form == "packed" else hermite)(p1, m1, p2, m2, fx)


def cases(seed, count):
    rng = np.random.default_rng(seed)
    for _ in range(count):
        n = int(rng.integers(2, 16))
        low, step = float(rng.uniform(-3, 0)), float(rng.uniform(0.2, 1.0))
        if rng.random() < 0.5:
            y = np.cumsum(rng.uniform(0, 0.4, n)) + 0.5   # monotone
        else:
            y = rng.normal(1.0, 0.5, n)                   # arbitrary shape
        xs = np.concatenate([low + step * np.arange(n),                         # on the knots
                             rng.uniform(low - 2 * n * step, low + 3 * n * step, 12)])
        yield low, step, y, xs


@pytest.mark.parametrize("dial_type", [MONOTONIC, COMPACT])
@pytest.mark.parametrize("form", ["prepared", "knots", "packed"])
def test_stored_forms_match_the_reference_in_fp64(dial_type, form):
    limit = dial_type == MONOTONIC
    worst = 0.0
    for low, step, y, xs in cases(7 + dial_type, 150):
        s = host_slopes(y, limit)
        scale = max(1.0, float(np.max(np.abs(y))))
        for trunc in (False, True):
            for x in xs:
                ref = O.dial(dial_type, np.concatenate([[low, step], y]), float(x), 0.0, trunc)
                got = evaluate(form, low, 1.0 / step, y, s, float(x), trunc, limit, float)
                worst = max(worst, abs(got - ref) / max(abs(ref), scale))
    assert worst <= 1e-12, worst


@pytest.mark.parametrize("dial_type", [MONOTONIC, COMPACT])
def test_knot_values_and_stored_slopes_give_the_same_fp64_value(dial_type):
    """The slopes formed on the device equal the host's, so the two stored
    forms evaluate to the same FP64 value (the engine's identical per-event
    weights)."""
    limit = dial_type == MONOTONIC
    for low, step, y, xs in cases(31 + dial_type, 100):
        s = host_slopes(y, limit)
        for x in xs:
            a = evaluate("prepared", low, 1.0 / step, y, s, float(x), False, limit, float)
            b = evaluate("knots", low, 1.0 / step, y, s, float(x), False, limit, float)
            assert a == b


@pytest.mark.parametrize("form", ["prepared", "knots", "packed"])
def test_stored_forms_in_fp32_arithmetic(form):
    """Within one knot step of the range (far extrapolation of a cubic
    cancels large terms and is ill-conditioned in FP32 for any form)."""
    f = np.float32
    worst = 0.0
    for low, step, y, xs in cases(101, 120):
        s = host_slopes(y, True)
        scale = max(1.0, float(np.max(np.abs(y))))
        xs = np.clip(xs, low - step, low + len(y) * step)
        for x in xs:
            ref = O.dial(MONOTONIC, np.concatenate([[low, step], y]), float(f(x)), 0.0, False)
            got = float(evaluate(form, f(low), f(1.0 / step), y.astype(f), s.astype(f), f(x), False, True, f))
            worst = max(worst, abs(got - ref) / max(abs(ref), scale))
    assert worst <= 2e-5, worst


# ---------------------------------------------------------------------------
# The coefficient form (GW_FLAG_SPLINE_COEFS) and the grid form
# (GW_FLAG_SPLINE_GRID), which evaluates the same blocks from an interval and
# fraction formed once per knot grid: write_prepared's per-interval cubics,
# the two extrapolation blocks re-expanded about their own origin, and
# coef_interval + the Horner cubic of eval_coef / the grid path.
# ---------------------------------------------------------------------------
UNIFORM = 3


def coef_blocks(y, sl, catmull):
    """write_prepared (coefficient / grid form): block j + 1 holds the cubic of
    u = xx - j on interval j; blocks 0 and n the extrapolation beyond the ends."""
    n = len(y)

    def cubic(i, m1, m2):
        dc = y[i + 1] - y[i]
        return [y[i], m1, 3.0 * dc - 2.0 * m1 - m2, m1 + m2 - 2.0 * dc]

    blocks = [None] * (n + 1)
    for j in range(n - 1):
        blocks[j + 1] = cubic(j, sl[j], sl[j + 1])
    c = cubic(0, sl[0], (y[1] - y[0]) if catmull else sl[1])
    blocks[0] = [c[0] - c[1] + c[2] - c[3], c[1] - 2.0 * c[2] + 3.0 * c[3], c[2] - 3.0 * c[3], c[3]]
    c = cubic(n - 2, (y[n - 1] - y[n - 2]) if catmull else sl[n - 2], sl[n - 1])
    blocks[n] = [c[0] + c[1] + c[2] + c[3], c[1] + 2.0 * c[2] + 3.0 * c[3], c[2] + 3.0 * c[3], c[3]]
    return blocks


def eval_coef(blocks, low, step, x, trunc, f):
    """coef_interval + coef_cubic: xx = x b + a, the truncation clamp,
    j = clamp(floor(xx), -1, n - 1), u = xx - j, block j + 1 at u."""
    n = len(blocks) - 1
    xx = f(x) * f(1.0 / step) + f(-low / step)
    if trunc:
        xx = min(max(xx, f(0)), f(n - 1))
    fj = min(max(f(math.floor(xx)), f(-1)), f(n - 1))
    u = xx - fj
    c = [f(q) for q in blocks[int(fj) + 1]]
    return c[0] + u * (c[1] + u * (c[2] + u * c[3]))


def uniform_cases(seed, count):
    rng = np.random.default_rng(seed)
    for low, step, y, xs in cases(seed, count):
        yield low, step, y, rng.normal(0.0, 0.5, len(y)), xs


@pytest.mark.parametrize("dial_type", [MONOTONIC, COMPACT, UNIFORM])
def test_coefficient_form_matches_the_reference_in_fp64(dial_type):
    """Within two knot steps of the range the re-expanded blocks reproduce the
    reference to 1e-12 of the knot scale; further out the extrapolated cubic
    grows as u^3 and the bound is taken on the value itself."""
    limit = dial_type == MONOTONIC
    worst = 0.0
    for low, step, y, dydx, xs in uniform_cases(211 + dial_type, 150):
        n = len(y)
        if dial_type == UNIFORM:
            data = np.concatenate([[low, step], np.stack([y, dydx], 1).ravel()])
            sl = dydx * step
        else:
            data = np.concatenate([[low, step], y])
            sl = host_slopes(y, limit)
        blocks = coef_blocks(y, sl, dial_type != UNIFORM)
        scale = max(1.0, float(np.max(np.abs(y))))
        for trunc in (False, True):
            for x in xs:
                ref = O.dial(dial_type, data, float(x), 0.0, trunc)
                got = eval_coef(blocks, low, step, float(x), trunc, float)
                near = low - 2 * step <= x <= low + (n + 1) * step
                worst = max(worst, abs(got - ref) / (max(abs(ref), scale) if near else max(abs(ref), 1.0)))
    assert worst <= 1e-12, worst


def test_coefficient_form_in_fp32_arithmetic():
    """FP32 blocks and interval within one knot step of the range, as the
    engine's FP32 mode evaluates them (the same bar as the other forms)."""
    f = np.float32
    worst = 0.0
    for low, step, y, xs in cases(307, 120):
        blocks = coef_blocks(y, host_slopes(y, True), True)
        scale = max(1.0, float(np.max(np.abs(y))))
        xs = np.clip(xs, low - step, low + len(y) * step)
        for x in xs:
            ref = O.dial(MONOTONIC, np.concatenate([[low, step], y]), float(f(x)), 0.0, False)
            got = float(eval_coef(blocks, low, step, f(x), False, f))
            worst = max(worst, abs(got - ref) / max(abs(ref), scale))
    assert worst <= 2e-5, worst
