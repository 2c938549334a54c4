"""The seeded workload generator: determinism and configuration shapes."""
import numpy as np

from gundam_gb300 import Workload
from gundam_gb300 import _native as N


def test_same_seed_same_workload_any_thread_count():
    a = Workload("mixed", seed=3, threads=1)
    b = Workload("mixed", seed=3, threads=8)
    for name in ("event_bin", "event_w0", "event_dial_start", "dial_type", "dial_par0", "dial_par1",
                 "dial_data_start", "dial_data", "data"):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)
    c = Workload("mixed", seed=4)
    assert not np.array_equal(a.dial_data[:100], c.dial_data[:100])


def test_c1_shape():
    w = Workload("c1", seed=1)
    assert w.n_events == 100000 and w.n_params == 22 and w.n_bins == 400
    assert np.all(np.diff(w.event_dial_start) == 5)
    t = w.dial_type.reshape(-1, 5)
    assert np.all(t[:, :3] == N.GW_DIAL_MONOTONIC) and np.all(t[:, 3:] == N.GW_DIAL_NORM)
    counts = np.bincount(w.event_bin, minlength=400)
    assert counts.min() > 150 and counts.max() < 350  # equal-probability binning
    # knots of every monotonic dial are monotone
    lens = np.diff(w.dial_data_start)
    mono = np.nonzero(w.dial_type == N.GW_DIAL_MONOTONIC)[0][:2000]
    for i in mono:
        y = w.dial_data[w.dial_data_start[i] + 2:w.dial_data_start[i] + lens[i]]
        d = np.diff(y)
        assert np.all(d >= 0) or np.all(d <= 0)


def test_c2_mix_at_reduced_size():
    w = Workload("c2", n_events=60000, seed=2)
    assert w.n_bins == 3000 and w.n_params == 200 and w.n_samples == 8
    nd = np.diff(w.event_dial_start)
    assert abs(nd.mean() - 8.0) < 0.1
    frac = np.bincount(w.dial_type, minlength=11)[1:8] / w.n_dials
    expect = {N.GW_DIAL_MONOTONIC: .5, N.GW_DIAL_UNIFORM: .2, N.GW_DIAL_GENERAL: .1, N.GW_DIAL_GRAPH: .1,
              N.GW_DIAL_BILINEAR: .05, N.GW_DIAL_NORM: .05}
    for t, f in expect.items():
        assert abs(frac[t - 1] - f) < 0.01, (t, frac[t - 1])
    # correlation-matrix prior (Wishart) on the spline parameters, unit diagonal
    c = w.prior_cov[:190, :190]
    assert np.allclose(np.diag(c), 1.0) and np.all(np.linalg.eigvalsh(c) > 0)


def test_mixed_has_every_dial_type_and_empty_bins():
    w = Workload("mixed", seed=5)
    assert set(np.unique(w.dial_type)) == set(range(1, 11))
    assert np.any(np.bincount(w.event_bin, minlength=w.n_bins) == 0)
    assert np.any(np.diff(w.event_dial_start) == 0)  # events without dials
    assert w.max_weight > 0 and w.n_tables == 2


def test_c2_algorithmic_bytes_match_the_per_dial_estimate():
    """The roofline numerator: the generated C2 mix stores ~15.35 reference
    values per dial (0.5*9 + 0.2*24 + 0.1*32 + 0.1*10 + 0.05*37), so one K = 1
    pass moves ~2.7 GB (FP32) / ~5.2 GB (FP64) at 5M events; the FP64 figure is
    the FP32 one plus 4 bytes per stored value and per event weight."""
    from gundam_gb300.roofline import algorithmic_bytes

    w = Workload("c2", n_events=100000, seed=2)
    lens = np.diff(w.dial_data_start)
    assert abs(lens.sum() / w.n_dials - 15.35) < 0.1
    b32, b64 = algorithmic_bytes(w, "fp32", 1), algorithmic_bytes(w, "fp64", 1)
    assert b64 - b32 == 4 * int(lens.sum()) + 4 * w.n_events
    per_event_scale = 5_000_000 / w.n_events
    assert 2.6e9 < b32 * per_event_scale < 2.9e9
    assert 5.0e9 < b64 * per_event_scale < 5.4e9
    # K points add only their parameters in and their bin sums out
    assert algorithmic_bytes(w, "fp32", 64) - b32 == 63 * (w.n_params * 8 + w.n_bins * 16)
