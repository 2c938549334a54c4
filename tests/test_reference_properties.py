"""The reference's own unit-test properties, restated against the oracle.

Sources: tests/GTests/unitTest_CalculateMonotonicSpline.cpp:15-153,
unitTest_DialDefinitions.cpp:22-250, unitTest_CalculateBilinearInterpolation.cpp:69-191,
unitTest_JointProbability.cpp:28-386 and cachedSumsTest.cpp:23-130 of the GUNDAM tree.
"""
import numpy as np
import pytest

from oracle import oracle as O

MONO, UNIF, GEN, COMP, GRAPH, BILIN, BICUB = 2, 3, 4, 5, 6, 7, 8


def test_monotonic_two_points_is_linear():
    d = [0.0, 1.0, 0.0, 1.0]
    for x in np.arange(-1.0, 2.0, 0.1):
        assert abs(O.dial(MONO, d, x) - x) < 1e-6


@pytest.mark.parametrize("ys", [
    [0.0, 1.0, 0.0],
    [0.0, 0.0, 1.0, 1.0, 0.0, 0.0],
    [0.5, 1.5, 1.0, 1.0, 1.0, 1.0, 0.5, 1.0, 1.0, 1.0, 1.0, 1.5, 0.5],
])
def test_monotonic_symmetric_knots_give_symmetric_curve(ys):
    n = len(ys)
    d = [-1.0, 2.0 / (n - 1), *ys]
    for x in np.arange(-1.1, 1.1, 0.01):
        assert abs(O.dial(MONO, d, x) - O.dial(MONO, d, -x)) < 1e-6


def test_monotonic_seventeen_cosine_knots_symmetric():
    n = 17
    xs = [-1.0 + i * 2.0 / (n - 1) for i in range(n)]
    d = [-1.0, 2.0 / (n - 1), *[np.cos(4.0 * x) for x in xs]]
    for x in np.arange(-1.1, 1.1, 0.01):
        assert abs(O.dial(MONO, d, x) - O.dial(MONO, d, -x)) < 1e-6


FIX_X = [-3.0, -2.0, -1.0, 0.0, 1.0, 2.0, 3.0]
FIX_Y = [1.75, 1.5, 1.0, 0.0, 1.0, 1.5, 1.75]


def _cr_slopes(x, y):
    n = len(x)
    s = [0.0] * n
    s[0] = (y[1] - y[0]) / (x[1] - x[0])
    s[-1] = (y[-1] - y[-2]) / (x[-1] - x[-2])
    for i in range(1, n - 1):
        s[i] = (y[i + 1] - y[i - 1]) / (x[i + 1] - x[i - 1])
    return s


def test_general_with_catmull_rom_slopes_equals_compact():
    s = _cr_slopes(FIX_X, FIX_Y)
    gen = [-3.0, 1.0, *[v for t in zip(FIX_Y, s, FIX_X) for v in t]]
    comp = [-3.0, 1.0, *FIX_Y]
    for x in np.arange(-3.0, 3.0, 0.05):
        assert abs(O.dial(GEN, gen, x) - O.dial(COMP, comp, x)) < 1e-9


def test_uniform_with_catmull_rom_slopes_equals_compact():
    s = _cr_slopes(FIX_X, FIX_Y)
    unif = [-3.0, 1.0, *[v for t in zip(FIX_Y, s) for v in t]]
    comp = [-3.0, 1.0, *FIX_Y]
    for x in np.arange(-3.0, 3.0, 0.05):
        assert abs(O.dial(UNIF, unif, x) - O.dial(COMP, comp, x)) < 1e-9


@pytest.mark.parametrize("t", [MONO, COMP])
def test_truncation_without_extrapolation(t):
    d = [-3.0, 1.0, *FIX_Y]
    assert O.dial(t, d, -10.0, truncate=True) == O.dial(t, d, -3.0)
    assert O.dial(t, d, 10.0, truncate=True) == O.dial(t, d, 3.0)
    assert O.dial(t, d, -10.0) != O.dial(t, d, -3.0)


def test_graph_end_values_without_extrapolation():
    g = [v for p in zip(FIX_Y, FIX_X) for v in p]
    assert O.dial(GRAPH, g, -5.0, truncate=True) == FIX_Y[0]
    assert O.dial(GRAPH, g, 5.0, truncate=True) == FIX_Y[-1]
    # extrapolation continues the end segments linearly
    assert abs(O.dial(GRAPH, g, -4.0) - 2.0) < 1e-12


@pytest.mark.parametrize("t", [BILIN, BICUB])
def test_surface_symmetry(t):
    g = [-1.0, 0.0, 1.0]
    z = [abs(a) + abs(b) for a in g for b in g]
    d = [3.0, 3.0, *g, *g, *z]
    for x in np.arange(-1.0, 1.0, 0.1):
        for y in np.arange(-1.0, 1.0, 0.1):
            v = O.dial(t, d, x, y)
            assert abs(v - O.dial(t, d, -x, y)) < 1e-8
            assert abs(v - O.dial(t, d, x, -y)) < 1e-8
            assert abs(v - O.dial(t, d, y, x)) < 1e-8


@pytest.mark.parametrize("llh", [1, 2])
def test_llh_continuous_and_minimal_at_data(llh):
    for data in (0.0, 1.0, 5.0, 50.0, 1000.0):
        preds = np.linspace(max(0.05, data * 0.5), data * 1.5 + 1.0, 400)
        vals = np.array([O.llh_bin(llh, data, p, np.sqrt(p) * 0.1) for p in preds])
        assert np.all(np.isfinite(vals))
        assert np.max(np.abs(np.diff(vals))) < 0.5 * (1 + data / 50)
        if llh == 1 and data > 0:
            i = int(np.argmin(vals))
            assert abs(preds[i] - data) <= (preds[1] - preds[0]) * 1.01
            assert abs(O.llh_bin(1, data, data, 0.0)) < 1e-9


def test_poisson_edge_values():
    assert O.llh_bin(1, 3.0, 0.0, 0.0) == float("inf")
    assert O.llh_bin(1, 0.0, 2.5, 0.0) == 5.0
    # Barlow-Beeston with no MC uncertainty is the Poisson statistic
    for d, p in ((3.0, 2.0), (10.0, 12.5)):
        assert abs(O.llh_bin(2, d, p, 0.0) - O.llh_bin(1, d, p, 0.0)) < 1e-12
    # with MC uncertainty it never exceeds the plain Poisson value
    for d, p in ((3.0, 2.0), (10.0, 12.5), (100.0, 80.0)):
        assert O.llh_bin(2, d, p, np.sqrt(p)) <= O.llh_bin(1, d, p, 0.0) + 1e-12
