"""CUDA engine against the FP64 CPU oracle on the same seeded inputs.

Tolerances (FP64 mode, as the acceptance bar states): per-bin relative error
<= 1e-12 on the sum of weights and the sum of squared weights, likelihood
absolute error <= 1e-6.  FP32 mode (dial math and weight product in FP32,
bins / sum of w^2 / likelihood in FP64): per-bin relative error <= 2e-5 and
likelihood absolute error <= 5e-2 (stated in FP32_* below).

Double-float mode (precision "df64": dial arithmetic and the weight product
in two-FP32-word numbers on the FP32 pipe, sums and likelihood in FP64) is
held to the FP64 bar above; its per-event weights to 1e-12 relative.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from gundam_gb300 import Engine, Workload
from gundam_gb300 import _native as N
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

FP64_BIN_REL = 1e-12
FP64_LLH_ABS = 1e-6
FP32_BIN_REL = 2e-5
FP32_LLH_ABS = 5e-2
# double-float mode (GW_DF64: dials and weight products in two-FP32-word
# arithmetic, ~48 significant bits; sums and likelihood in FP64) is held to
# the FP64 bar; its per-event weights carry a few 2^-48 of rounding
DF64_EVENT_REL = 1e-12


def _tol(precision):
    return (FP32_BIN_REL, FP32_LLH_ABS) if precision == "fp32" else (FP64_BIN_REL, FP64_LLH_ABS)


def _bin_rel(got, ref):
    got, ref = np.asarray(got), np.asarray(ref)
    den = np.where(ref != 0, np.abs(ref), 1.0)
    return float(np.max(np.abs(got - ref) / den))


def _check(eng_out, orc, bin_rel, llh_abs, label=""):
    sums, sums2, llh, stat = eng_out
    assert _bin_rel(sums, orc["sums"]) <= bin_rel, label
    assert _bin_rel(sums2, orc["sums2"]) <= bin_rel, label
    fin = np.isfinite(orc["llh"])
    assert np.array_equal(np.isfinite(llh), fin), label
    assert np.max(np.abs(llh[fin] - orc["llh"][fin]), initial=0.0) <= llh_abs, label
    assert np.max(np.abs(stat[fin] - orc["llh_stat"][fin]), initial=0.0) <= llh_abs, label


@pytest.fixture(scope="module")
def c1():
    return Workload("c1", seed=11)


@pytest.fixture(scope="module")
def c1_oracle(c1):
    return Oracle(c1, llh_type=N.GW_LLH_POISSON)


@pytest.fixture(scope="module")
def mixed():
    return Workload("mixed", seed=5)


@pytest.fixture(scope="module")
def mixed_oracle(mixed):
    return Oracle(mixed, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021)


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_c1_plain(c1, c1_oracle, precision):
    eng = Engine.from_workload(c1, precision=precision, k_max=1, llh_type=N.GW_LLH_POISSON)
    pts = np.vstack([c1.nominal(), c1.draw_points(24, 5)])
    for i, p in enumerate(pts):
        _check(eng.eval(p[None]), c1_oracle.eval(p[None]), FP64_BIN_REL, FP64_LLH_ABS, f"point {i}")
    eng.close()


def test_c1_fp32_plain(c1, c1_oracle):
    eng = Engine.from_workload(c1, precision="fp32", k_max=1, llh_type=N.GW_LLH_POISSON)
    pts = np.vstack([c1.nominal(), c1.draw_points(12, 6)])
    for i, p in enumerate(pts):
        _check(eng.eval(p[None]), c1_oracle.eval(p[None]), FP32_BIN_REL, FP32_LLH_ABS, f"point {i}")
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_c1_thousand_points(c1, c1_oracle, precision):
    """C1's stated result: Poisson LLH and bin contents at 1000 random
    parameter points, in four batched launches of 250 points."""
    eng = Engine.from_workload(c1, precision=precision, k_max=250, llh_type=N.GW_LLH_POISSON)
    pts = c1.draw_points(1000, 1000)
    ref = c1_oracle.eval(pts)
    parts = [eng.eval(pts[a:a + 250]) for a in range(0, 1000, 250)]
    out = tuple(np.concatenate([p[i] for p in parts]) for i in range(4))
    _check(out, ref, FP64_BIN_REL, FP64_LLH_ABS, "1000 points")
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32", "df64"])
@pytest.mark.parametrize("K", [2, 4, 16, 64, 200, 256])
def test_c1_batched(c1, c1_oracle, precision, K):
    eng = Engine.from_workload(c1, precision=precision, k_max=256, llh_type=N.GW_LLH_POISSON)
    pts = c1.draw_points(K, 100 + K)
    ref = c1_oracle.eval(pts)
    rel, ab = _tol(precision)
    _check(eng.eval(pts), ref, rel, ab, f"K={K}")
    eng.close()


def test_batched_point_equals_plain_point(c1):
    """Point k of a batch gives the same bins as evaluating it alone (FP64)."""
    eng = Engine.from_workload(c1, precision="fp64", k_max=64)
    pts = c1.draw_points(64, 77)
    sb, s2b, lb, _ = eng.eval(pts)
    for k in (0, 17, 63):
        s, s2, l, _ = eng.eval(pts[k:k + 1])
        assert _bin_rel(sb[k], s[0]) <= FP64_BIN_REL
        assert abs(lb[k] - l[0]) <= FP64_LLH_ABS
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_mixed_all_dial_types(mixed, mixed_oracle, precision):
    """Every dial type, mirrored and truncated parameters, response clamps, the
    weight cap, host tables, base weights != 1, events without dials and empty bins."""
    eng = Engine.from_workload(mixed, precision=precision, k_max=8, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021)
    eng.set_event_weight_copy(True)
    pts = np.vstack([mixed.nominal(), mixed.draw_points(15, 9, inflate=1.6)])
    for i, p in enumerate(pts):
        ref = mixed_oracle.eval(p[None], weights=True)
        out = eng.eval(p[None])
        _check(out, ref, FP64_BIN_REL, FP64_LLH_ABS, f"point {i}")
        w = eng.event_weights()
        assert _bin_rel(w, ref["weights"]) <= (1e-13 if precision == "fp64" else DF64_EVENT_REL)
        counts = np.bincount(mixed.event_bin, minlength=mixed.n_bins)
        assert np.any(counts == 0) and np.all(out[0][0][counts == 0] == 0.0)
    _check(eng.eval(pts[:8]), mixed_oracle.eval(pts[:8]), FP64_BIN_REL, FP64_LLH_ABS, "batched")
    eng.close()


def test_mixed_fp32(mixed, mixed_oracle):
    eng = Engine.from_workload(mixed, precision="fp32", k_max=8, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021)
    pts = mixed.draw_points(8, 19, inflate=1.4)
    _check(eng.eval(pts), mixed_oracle.eval(pts), FP32_BIN_REL, FP32_LLH_ABS)
    eng.close()


def test_per_dial_api_equals_batched_api(mixed):
    a = Engine.from_workload(mixed, precision="fp64", k_max=4)
    b = Engine.from_workload(mixed, precision="fp64", k_max=4, per_dial=True)
    pts = mixed.draw_points(4, 3)
    ra, rb = a.eval(pts), b.eval(pts)
    for x, y in zip(ra, rb):
        np.testing.assert_array_equal(x, y)
    a.close()
    b.close()


def test_graph_capture_gives_identical_results(c1):
    eng = Engine.from_workload(c1, precision="fp32", k_max=64)
    pts = c1.draw_points(64, 8)
    plain = [eng.eval(pts), eng.eval(pts[:1])]
    eng.use_graph(True)
    graph = [eng.eval(pts), eng.eval(pts[:1]), eng.eval(pts)]
    for x, y in zip(plain[0], graph[0]):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(plain[1], graph[1]):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(graph[0], graph[2]):
        np.testing.assert_array_equal(x, y)
    eng.close()


def test_device_path_graph_replay_matches_direct_launch(c1):
    """gw_eval_device with graphs on: the captured chain replayed on the
    caller's stream gives the same bits as the direct launches, also after
    new parameters are written into the same device buffer."""
    import torch
    eng = Engine.from_workload(c1, precision="fp32", k_max=64)
    K = 48
    stream = torch.cuda.Stream()
    p = torch.from_numpy(c1.draw_points(K, 21)).cuda()
    outs = [torch.empty((K, c1.n_bins), dtype=torch.float64, device="cuda") for _ in range(2)]
    ll = torch.empty(K, dtype=torch.float64, device="cuda")

    def run():
        eng.eval_device(p.data_ptr(), K, outs[0].data_ptr(), outs[1].data_ptr(), ll.data_ptr(), 0,
                        stream.cuda_stream)
        stream.synchronize()
        return [o.cpu().numpy().copy() for o in outs] + [ll.cpu().numpy().copy()]
    direct = run()
    eng.use_graph(True)
    g1, g2 = run(), run()
    for x, y, z in zip(direct, g1, g2):
        np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(x, z)
    p.copy_(torch.from_numpy(c1.draw_points(K, 22)))
    g3 = run()
    eng.use_graph(False)
    d3 = run()
    for x, y in zip(g3, d3):
        np.testing.assert_array_equal(x, y)
    assert not np.array_equal(g3[2], direct[2])
    eng.close()


def test_results_are_deterministic(c1):
    eng = Engine.from_workload(c1, precision="fp64", k_max=32)
    pts = c1.draw_points(32, 4)
    r1, r2 = eng.eval(pts), eng.eval(pts)
    for x, y in zip(r1, r2):
        np.testing.assert_array_equal(x, y)
    eng.close()


def test_autotune_picks_a_valid_shape(c1, c1_oracle):
    eng = Engine.from_workload(c1, precision="fp32", k_max=64)
    eng.autotune(64)
    kind, kc, th, st = eng.shape()
    assert kind in (0, 1, 3) and kc in (2, 4, 8, 16, 32, 64, 128) and th in (128, 256) and st in (1, 2)
    pts = c1.draw_points(64, 12)
    _check(eng.eval(pts), c1_oracle.eval(pts), FP32_BIN_REL, FP32_LLH_ABS)
    eng.close()


def test_event_weights_c1(c1, c1_oracle):
    eng = Engine.from_workload(c1, precision="fp64", k_max=1)
    eng.set_event_weight_copy(True)
    p = c1.draw_points(1, 55)
    eng.eval(p)
    w = eng.event_weights()
    ref = c1_oracle.eval(p, weights=True)["weights"]
    assert _bin_rel(w, ref) <= 1e-13
    eng.close()


GOLDEN = json.loads((Path(__file__).parent / "golden" / "dials.json").read_text())


def _extrapolation_factor(t, d, x, y):
    """(1 + distance outside the knot range, in knot steps)^3: how much a cubic
    extrapolation amplifies one rounding difference (FMA vs. separate multiply
    and add on the device)."""
    def far(v, xs):
        xs = np.asarray(xs, dtype=float)
        if len(xs) < 2:
            return 0.0
        step = float(np.min(np.diff(xs)))
        return max(0.0, (xs[0] - v) / step, (v - xs[-1]) / step)

    d = np.asarray(d, dtype=float)
    if t in (2, 5):
        n = len(d) - 2
        return (1 + far(x, d[0] + d[1] * np.arange(n))) ** 3
    if t == 3:
        n = (len(d) - 2) // 2
        return (1 + far(x, d[0] + d[1] * np.arange(n))) ** 3
    if t == 4:
        return (1 + far(x, d[4::3])) ** 3
    if t == 6:
        return 1 + far(x, d[1::2])
    nx, ny = int(d[0]), int(d[1])
    fx, fy = far(x, d[2:2 + nx]), far(y, d[2 + nx:2 + nx + ny])
    return ((1 + fx) * (1 + fy)) ** 3


@pytest.mark.parametrize("precision", ["fp64", "fp32", "df64"])
def test_reference_golden_dials_through_engine(precision):
    """One event per golden case, one dial per event, on its own parameter(s);
    the event weight is the dial response computed by the reference's own
    Calculate*.h."""
    data = GOLDEN["data"]
    cases = [c for c in GOLDEN["cases"] if abs(c[4]) < 1e19]
    n = len(cases)
    chunk = 2000
    for s in range(0, n, chunk):
        part = cases[s:s + chunk]
        m = len(part)
        P = 2 * m
        eng = Engine(m, P, 1, k_max=1, precision=precision)
        params = np.zeros(P)
        for p in range(P):
            eng.set_lower_clamp(p, -np.finfo(np.float64).max)
        for i, (t, di, x, y, v) in enumerate(part):
            d = data[di]
            if t in (7, 8):
                eng.add_surface(t, i, 2 * i, 2 * i + 1, d)
            elif t == 6:
                eng.add_graph(i, 2 * i, d)
            else:
                eng.add_spline(t, i, 2 * i, d)
            params[2 * i] = x
            params[2 * i + 1] = y
        eng.set_event_indices(np.zeros(m, dtype=np.int32))
        eng.initialize()
        eng.set_event_weight_copy(True)
        eng.eval(params[None])
        w = eng.event_weights()
        ref = np.array([c[4] for c in part])
        amp = np.array([_extrapolation_factor(c[0], data[c[1]], c[2], c[3]) for c in part])
        if precision == "fp64":
            tol = 1e-13 * np.maximum(1.0, np.abs(ref)) * amp
        elif precision == "df64":
            tol = 1e-12 * np.maximum(1.0, np.abs(ref)) * amp
        else:
            tol = 1e-4 * np.maximum(1.0, np.abs(ref)) * amp
        bad = np.nonzero(np.abs(w - ref) > tol)[0]
        assert bad.size == 0, [(part[i][0], part[i][2], part[i][3], ref[i], w[i]) for i in bad[:5]]
        eng.close()


def test_c2_subset_all_precisions():
    wl = Workload("c2", n_events=300000, seed=21)
    orc = Oracle(wl, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021)
    pts = np.vstack([wl.nominal(), wl.draw_points(5, 2)])
    ref = orc.eval(pts)
    e64 = Engine.from_workload(wl, precision="fp64", k_max=8)
    _check(e64.eval(pts), ref, FP64_BIN_REL, FP64_LLH_ABS, "c2 fp64 batched")
    for i in range(2):
        _check(e64.eval(pts[i:i + 1]), orc.eval(pts[i:i + 1]), FP64_BIN_REL, FP64_LLH_ABS, "c2 fp64 plain")
    e64.close()
    e32 = Engine.from_workload(wl, precision="fp32", k_max=8)
    _check(e32.eval(pts), ref, FP32_BIN_REL, FP32_LLH_ABS, "c2 fp32")
    e32.close()
    edf = Engine.from_workload(wl, precision="df64", k_max=8)
    _check(edf.eval(pts), ref, FP64_BIN_REL, FP64_LLH_ABS, "c2 df64 batched")
    for i in range(2):
        _check(edf.eval(pts[i:i + 1]), orc.eval(pts[i:i + 1]), FP64_BIN_REL, FP64_LLH_ABS, "c2 df64 plain")
    edf.close()


def test_device_pointer_entry_point(c1, c1_oracle):
    torch = pytest.importorskip("torch")
    eng = Engine.from_workload(c1, precision="fp64", k_max=16)
    pts = c1.draw_points(16, 31)
    d_p = torch.from_numpy(pts).cuda()
    d_s = torch.empty((16, c1.n_bins), dtype=torch.float64, device="cuda")
    d_s2 = torch.empty_like(d_s)
    d_l = torch.empty(16, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    eng.eval_device(d_p.data_ptr(), 16, d_s.data_ptr(), d_s2.data_ptr(), d_l.data_ptr(), 0, stream)
    torch.cuda.synchronize()
    eng.sync()
    ref = c1_oracle.eval(pts)
    assert _bin_rel(d_s.cpu().numpy(), ref["sums"]) <= FP64_BIN_REL
    assert np.max(np.abs(d_l.cpu().numpy() - ref["llh"])) <= FP64_LLH_ABS
    eng.close()


@pytest.mark.parametrize("name,cfg,events", [("c1", "c1", 0), ("c2s", "c2", 20000)])
def test_engine_matches_reference_cache_manager_fixtures(name, cfg, events):
    """Per-bin sums of the engine (FP64 and FP32 modes) against GUNDAM's own
    Cache::Manager calculators (tests/golden/cache_sums.npz); empty bins are
    0 here and the next bin's content there (documented difference)."""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "cache_sums.npz")
    wl = Workload(cfg, n_events=events, seed=2)
    pts = g[f"{name}_points"]
    occ = np.bincount(wl.event_bin, minlength=wl.n_bins) > 0
    for prec, tol in (("fp64", 1e-12), ("fp32", 2e-5), ("df64", 1e-12)):
        eng = Engine.from_workload(wl, precision=prec, k_max=len(pts))
        s, s2, _, _ = eng.eval(pts)
        for got, ref in ((s, g[f"{name}_sums"]), (s2, g[f"{name}_sums2"])):
            rel = np.abs(got - ref)[:, occ] / np.abs(ref[:, occ])
            assert rel.max() < tol, (name, prec, rel.max())
            assert np.all(got[:, ~occ] == 0.0)
        eng.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32", "df64"])
def test_all_k1_kernels_agree_bit_for_bit(mixed, prec):
    """k_plain and the warp-specialised k_plain_ws (six or eight evaluator
    warps) form the same products and sums in the same order: identical
    results, per-event weights included; gw_autotune(1) picks one of them."""
    eng = Engine.from_workload(mixed, precision=prec, k_max=4)
    eng.set_event_weight_copy(True)
    pt = mixed.draw_points(1, 41)
    out = []
    for kind in (0, 1, 2):
        eng.set_plain_kernel(kind)
        assert eng.plain_kernel() == kind
        r = eng.eval(pt)
        out.append([np.array(x, copy=True) for x in r] + [eng.event_weights().copy()])
    for other in out[1:]:
        for x, y in zip(out[0], other):
            np.testing.assert_array_equal(x, y)
    eng.autotune(1)
    assert eng.plain_kernel() in (0, 1, 2)
    r = eng.eval(pt)
    np.testing.assert_array_equal(r[0], out[0][0])
    eng.close()


def test_eigen_decomposed_parameters(c1, c1_oracle):
    """Parameters given in the eigen basis of the prior covariance (original =
    V * eigen on the device) reproduce the oracle at the original values; a
    diagonal prior on the eigen parameters gives the original penalty."""
    lam, V = np.linalg.eigh(c1.prior_cov)
    # the cache with one eigen block over all parameters and the eigen-space prior
    e2 = Engine.from_workload(c1, precision="fp64", k_max=8, prior=False, initialize=False)
    e2.add_eigen_block(0, V)
    e2.set_prior(V.T @ c1.prior_mean, np.diag(1.0 / lam))
    e2.initialize()
    x = c1.draw_points(8, 91)
    y = x @ V  # eigen = V^T x, row-wise
    s, s2, llh, stat = e2.eval(y)
    r = c1_oracle.eval(x)
    np.testing.assert_allclose(s, r["sums"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(s2, r["sums2"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(stat, r["llh_stat"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(llh, r["llh"], rtol=1e-10, atol=1e-6)
    e2.close()


@pytest.mark.parametrize("prec,layout", [("fp64", "auto"), ("fp32", "auto"), ("df64", "auto"), ("fp32", "coefs"),
                                         ("fp64", "coefs"), ("fp32", "slopes"), ("df64", "slopes")])
def test_every_compiled_batched_shape(mixed, mixed_oracle, prec, layout):
    """Every compiled batched kernel shape (every family, every register
    target) on the workload with every dial type, K = 64 inflated prior draws
    (extrapolation beyond the knot ranges included), against the oracle; the
    register targets of one shape give identical results.  Also with the
    uniform-knot splines in the grid form (the default at k_max = 64: the
    coefficients with the knot grid's interval formed once per point), the
    coefficient form and the slope form."""
    K = 64
    eng = Engine.from_workload(mixed, precision=prec, k_max=K, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021,
                               spline_layout=layout)
    pts = mixed.draw_points(K, 77, inflate=2.5)
    ref = mixed_oracle.eval(pts)
    tol = _tol(prec)
    first = {}
    tried = 0
    for i, (kind, ppp, ppt, threads, stages, minb) in enumerate(Engine.compiled_shapes()):
        if ppp > K:
            continue  # a 128-point pass would run past the engine's 64 padded point columns
        try:
            eng.set_shape_index(i)
        except RuntimeError:
            continue  # does not fit on an SM at this tile size
        assert eng.shape_index() == i and eng.shape() == (kind, ppp, threads, stages)
        out = [np.array(x, copy=True) for x in eng.eval(pts)]
        _check(out, ref, *tol, f"shape {(kind, ppp, ppt, threads, stages, minb)}")
        key = (kind, ppp, ppt, threads, stages)
        if key in first:
            for x, y in zip(first[key], out):
                np.testing.assert_array_equal(x, y)
        else:
            first[key] = out
        tried += 1
    assert tried >= (5 if prec == "df64" else 10)  # double-float is compiled for five shapes
    eng.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_wide_shapes_at_256_points(mixed, mixed_oracle, prec):
    """The lanes shapes of 128 points per pass (four points per lane, the
    grid-form table entries loaded one dial ahead) at K = 256 on the workload
    with every dial type, grid form (the default at k_max = 256), inflated
    prior draws: each against the oracle."""
    K = 256
    eng = Engine.from_workload(mixed, precision=prec, k_max=K, llh_type=N.GW_LLH_BARLOW_BEESTON_OA2021)
    pts = mixed.draw_points(K, 78, inflate=2.5)
    ref = mixed_oracle.eval(pts)
    tried = 0
    for i, (kind, ppp, ppt, threads, stages, minb) in enumerate(Engine.compiled_shapes()):
        if kind != 0 or ppp != 128:
            continue
        try:
            eng.set_shape_index(i)
        except RuntimeError:
            continue
        _check(eng.eval(pts), ref, *_tol(prec), f"shape {(kind, ppp, ppt, threads, stages, minb)}")
        tried += 1
    assert tried >= 2
    eng.close()


def test_shape_that_overruns_the_padded_points_is_refused(c1, c1_oracle):
    """K = 150 pads to 192 point columns: a 128-point pass would need 256, so
    the launch is refused with an error (never a read past the arrays); the
    autotuner only picks shapes that fit, and those agree with the oracle."""
    K = 150
    eng = Engine.from_workload(c1, precision="fp32", k_max=K, llh_type=N.GW_LLH_POISSON)
    pts = c1.draw_points(K, 21)
    eng.set_shape(0, 128, 128, 1)
    with pytest.raises(N.GwError, match="does not cover"):
        eng.eval(pts)
    eng.autotune(K)
    kind, ppp, _, _ = eng.shape()
    assert ppp <= 64 or kind == 1
    _check(eng.eval(pts), c1_oracle.eval(pts), FP32_BIN_REL, FP32_LLH_ABS)
    eng.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_spline_layouts_agree(mixed, mixed_oracle, prec):
    """Catmull-Rom splines stored as knot values (the slopes formed on the
    device), with slopes precomputed on the host, or all uniform-knot splines
    as per-interval cubic coefficients (extrapolation intervals included):
    each within tolerance of the oracle through the K = 1 and the batched
    kernels, with draws far enough out to extrapolate.  In FP64 the knot and
    slope forms give identical per-event weights, and so do the coefficient
    and grid forms in both precisions; the bin sums differ only in
    rounding, because the smaller payload cuts different tiles and so groups
    the FP64 partial sums differently.  The knot form packs fewer bytes, and
    an FP32 K = 1 engine picks it."""
    llh = N.GW_LLH_BARLOW_BEESTON_OA2021
    pts = mixed.draw_points(4, 61, inflate=2.0)
    ref = mixed_oracle.eval(pts)
    tol = (FP64_BIN_REL, FP64_LLH_ABS) if prec == "fp64" else (FP32_BIN_REL, FP32_LLH_ABS)
    out = {}
    for layout in ("knots", "slopes", "coefs", "grid"):
        eng = Engine.from_workload(mixed, precision=prec, k_max=4, llh_type=llh, spline_layout=layout)
        eng.set_event_weight_copy(True)
        weights = []
        for i in range(len(pts)):
            r = eng.eval(pts[i:i + 1])
            _check(r, {k: ref[k][i:i + 1] for k in ref}, *tol, f"{layout} K=1 point {i}")
            weights.append(eng.event_weights().copy())
        _check(eng.eval(pts), ref, *tol, f"{layout} K=4")
        out[layout] = (weights, eng.layout()["payload_bytes"])
        eng.close()
    if prec == "fp64":
        for wk, ws in zip(out["knots"][0], out["slopes"][0]):
            np.testing.assert_array_equal(wk, ws)
    # the grid form evaluates the same cubic from the same interval: identical
    # per-event weights in either precision, four fewer values per spline
    for wc, wg in zip(out["coefs"][0], out["grid"][0]):
        np.testing.assert_array_equal(wc, wg)
    assert out["grid"][1] < out["coefs"][1]
    assert out["knots"][1] < out["slopes"][1]
    auto = Engine.from_workload(mixed, precision=prec, k_max=1, llh_type=llh)
    assert auto.layout()["payload_bytes"] == out["knots" if prec == "fp32" else "slopes"][1]
    auto.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_grid_form_beyond_the_grid_limit(prec):
    """More distinct knot grids than the grid form holds (16384): the splines
    of the grids past the limit keep the coefficient form in the same engine.
    Every spline here has its own step, and three in four share their
    parameter with others; per-event weights through the K = 1 kernel equal
    the coefficient form's, and the batched sums agree within rounding."""
    rng = np.random.default_rng(5)
    n_ev, P, B = 20000, 50, 40
    knots = 7
    types, res, p0, starts, data = [], [], [], [0], []
    for i in range(n_ev):
        step = 0.5 + 1e-4 * i  # a grid per spline
        y = np.exp(np.cumsum(rng.normal(0.0, 0.05, knots)))
        d = np.concatenate([[-3.0, step], y])
        for t, pp in ((N.GW_DIAL_MONOTONIC, i % P), (N.GW_DIAL_UNIFORM, (7 * i) % P)):
            if t == N.GW_DIAL_UNIFORM:
                d = np.concatenate([[-3.0, step], np.stack([y, rng.normal(0.0, 0.1, knots)], 1).ravel()])
            types.append(t)
            res.append(i)
            p0.append(pp)
            data.append(d)
            starts.append(starts[-1] + len(d))
    bins = rng.integers(0, B, n_ev)
    pts = rng.normal(0.0, 1.5, (4, P))
    out = {}
    for layout in ("coefs", "grid"):
        e = Engine(n_ev, P, B, k_max=4, precision=prec, spline_layout=layout)
        e.set_initial_values(np.full(n_ev, 1.0))
        e.set_event_indices(bins)
        e.add_dials(np.array(types), np.array(res), np.array(p0), np.full(len(types), -1),
                    np.array(starts), np.concatenate(data))
        e.set_data(np.full(B, 500.0))
        e.set_likelihood(N.GW_LLH_POISSON)
        e.initialize()
        e.set_event_weight_copy(True)
        w = []
        for k in range(len(pts)):
            e.eval(pts[k:k + 1])
            w.append(e.event_weights().copy())
        out[layout] = (w, e.eval(pts), e.layout()["payload_bytes"])
        e.close()
    for a, b in zip(out["coefs"][0], out["grid"][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_allclose(out["grid"][1][0], out["coefs"][1][0], rtol=1e-12 if prec == "fp64" else 1e-6)
    # 16384 splines lose their four-value prefix, the others keep it
    tsz = 8 if prec == "fp64" else 4
    saved = out["coefs"][2] - out["grid"][2]
    assert 0.9 * 16384 * 4 * tsz <= saved <= 1.1 * 16384 * 4 * tsz + 16 * 2000
