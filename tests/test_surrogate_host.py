"""Host-side pieces of the surrogate (CPU): the base's design matrix and its
ridge fit, the Σw² model and the learning-rate schedule.  The network and the
device head are exercised by the GPU tests."""
import math

import numpy as np

from gundam_gb300.surrogate import Surrogate, cosine_lr


def _host_surrogate(n_params, n_bins):
    """A Surrogate without its device network: only the host-side fit."""
    s = Surrogate.__new__(Surrogate)
    s.n_params, s.n_bins = n_params, n_bins
    s.kind, s.nodes, s.lim = "affine", 0, 0.0
    s.rb = s.rw = None
    s.seed = 0
    return s


def test_cosine_schedule_end_points():
    assert cosine_lr(0, 100, 1e-3) == 1e-3
    assert math.isclose(cosine_lr(50, 100, 1e-3, 1e-5), 0.5 * (1e-3 + 1e-5))
    assert math.isclose(cosine_lr(100, 100, 1e-3, 1e-5), 1e-5)
    assert math.isclose(cosine_lr(250, 100, 1e-3, 1e-5), 1e-5)  # held after the end


def test_additive_features_are_a_partition_of_unity_per_parameter():
    s = _host_surrogate(5, 3)
    s.kind, s.nodes, s.lim = "additive", 8, 3.0
    z = np.random.default_rng(1).normal(0, 2.0, (200, 5))  # some beyond +-lim
    F = s._features(z)
    assert F.shape == (200, 1 + 5 * 8)
    assert np.all(F[:, 0] == 1.0)
    per_param = F[:, 1:].reshape(200, 5, 8).sum(axis=2)
    np.testing.assert_allclose(per_param, 1.0, atol=1e-12)
    assert np.all(F >= 0.0)


def test_affine_base_reproduces_affine_rates():
    rng = np.random.default_rng(2)
    P, B, n = 6, 4, 500
    th = rng.normal(0.3, 0.8, (n, P))
    W, c = rng.normal(0, 0.2, (P, B)), rng.normal(3, 1, B)
    logs = c + th @ W
    s = _host_surrogate(P, B)
    resid = s.fit_affine(th, logs)
    assert np.max(np.abs(resid)) < 1e-8
    np.testing.assert_allclose(s.base(th[:7]), logs[:7], atol=1e-8)
    assert np.all(s.r_sd == 1.0)  # exactly reproduced bins keep unit scale


def test_additive_base_reproduces_additive_rates_and_the_ratio_model():
    """Rates that are a sum of per-parameter piecewise-linear functions on the
    base's own nodes are reproduced (up to the ridge term); log(Σw²/Σw) is
    fitted as an affine function."""
    rng = np.random.default_rng(3)
    P, B, n = 4, 3, 4000
    th = rng.normal(0.0, 1.0, (n, P))
    s = _host_surrogate(P, B)
    s.kind, s.nodes, s.lim = "additive", 8, 3.0
    s.mu, s.sd = th.mean(axis=0), th.std(axis=0) + 1e-12
    F = s._features(s._z(th))
    A_true = rng.normal(0, 0.3, (F.shape[1], B))
    logs = F @ A_true
    R_true = rng.normal(0, 0.1, (1 + P, B))
    log_ratio = np.hstack([np.ones((n, 1)), s._z(th)]) @ R_true
    resid = s.fit_additive(th, logs, log_ratio=log_ratio, nodes=8, lim=3.0, ridge=1e-10)
    assert np.max(np.abs(resid)) < 1e-5
    np.testing.assert_allclose(s.rb, R_true[0], atol=1e-8)
    np.testing.assert_allclose(s.rw, R_true[1:].T, atol=1e-8)
