"""Samplers on an analytic Gaussian target (CPU): plain and delayed
acceptance recover the posterior, and delayed acceptance with an imperfect
surrogate stays exact (the surrogate only changes efficiency)."""
import numpy as np

from gundam_gb300 import mcmc


def _target(P=6, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((P, P))
    cov = A @ A.T / P + 0.5 * np.eye(P)
    mean = rng.standard_normal(P)
    icov = np.linalg.inv(cov)

    def f(th):
        d = th - mean
        return np.einsum("ij,jk,ik->i", d, icov, d)
    return mean, cov, icov, f


def test_plain_recovers_gaussian():
    mean, cov, icov, f = _target()
    L = mcmc.proposal_chol(cov)
    r = mcmc.plain(f, np.tile(mean, (32, 1)), 3000, L, seed=1)
    x = r["chains"][500:].reshape(-1, mean.size)
    assert np.allclose(x.mean(0), mean, atol=0.1)
    assert np.allclose(x.std(0), np.sqrt(np.diag(cov)), rtol=0.1)
    assert 0.15 < r["accept"] < 0.5


def test_delayed_acceptance_is_exact_with_a_biased_surrogate():
    mean, cov, icov, f = _target()
    shift = 0.3 * np.sqrt(np.diag(cov))
    icov_s = np.linalg.inv(1.3 * cov)

    def f_sur(th):  # wrong mean and width
        d = th - mean - shift
        return np.einsum("ij,jk,ik->i", d, icov_s, d)
    L = mcmc.proposal_chol(cov)
    r = mcmc.delayed(f, f_sur, np.tile(mean, (32, 1)), 2500, L, n_sub=5, seed=2, max_error=1e9)
    x = r["chains"][300:].reshape(-1, mean.size)
    assert np.allclose(x.mean(0), mean, atol=0.12)
    assert np.allclose(x.std(0), np.sqrt(np.diag(cov)), rtol=0.12)
    assert r["fell_back_at_step"] is None


def test_delayed_with_good_surrogate_gains_ess_per_exact_evaluation():
    mean, cov, icov, f = _target()
    L = mcmc.proposal_chol(cov)
    th0 = np.tile(mean, (32, 1))
    p = mcmc.plain(f, th0, 1500, L, seed=3)
    d = mcmc.delayed(f, f, th0, 1500, L, n_sub=8, seed=4)
    ess_p = mcmc.ess(p["chains"], burn=200).min() / p["n_exact"]
    ess_d = mcmc.ess(d["chains"], burn=200).min() / d["n_exact"]
    assert d["stage2_accept"] > 0.99  # exact surrogate: stage 2 always agrees
    assert ess_d > 3 * ess_p


def test_fallback_when_surrogate_error_grows():
    mean, cov, icov, f = _target()
    L = mcmc.proposal_chol(cov)

    noise = np.random.default_rng(9)

    def bad(th):  # disagrees with the target by ~10 units of -2 log L
        return f(th) + noise.normal(0.0, 10.0, th.shape[0])
    r = mcmc.delayed(f, bad, np.tile(mean, (16, 1)), 200, L, n_sub=4, seed=5, max_error=5.0)
    assert r["fell_back_at_step"] is not None


def test_frozen_fallback_runs_plain_from_the_first_step_or_never_switches():
    """The fall-back decided in a warm-up is frozen for the recorded run:
    start_plain makes every step a plain step (the surrogate is never
    called), max_error = inf never switches whatever the error."""
    mean, cov, icov, f = _target()
    L = mcmc.proposal_chol(cov)

    def never(th):
        raise AssertionError("surrogate called in a plain run")
    r = mcmc.delayed(f, never, np.tile(mean, (8, 1)), 50, L, n_sub=4, seed=5, start_plain=True)
    assert r["fell_back_at_step"] == 0 and r["n_surrogate"] == 8
    noise = np.random.default_rng(9)

    def bad(th):
        return f(th) + noise.normal(0.0, 10.0, th.shape[0])
    r = mcmc.delayed(f, bad, np.tile(mean, (16, 1)), 200, L, n_sub=4, seed=5, max_error=float("inf"))
    assert r["fell_back_at_step"] is None


def test_ess_of_independent_draws_is_close_to_n():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((4000, 4, 3))
    e = mcmc.ess(x)
    assert np.all(e > 0.8 * 16000) and np.all(e < 1.2 * 16000)


def test_delayed_with_hmc_stage1_is_exact_with_a_biased_surrogate():
    """Hamiltonian stage 1 on a wrong surrogate (shifted mean, wider
    covariance) still samples the exact target after the stage-2 correction,
    and with a good surrogate its proposals are far apart (large ESS per
    exact evaluation)."""
    mean, cov, icov, f = _target()
    shift = 0.3 * np.sqrt(np.diag(cov))
    icov_s = np.linalg.inv(1.3 * cov)

    def vg_bad(th):
        d = th - mean - shift
        return np.einsum("ij,jk,ik->i", d, icov_s, d), 2.0 * d @ icov_s

    Lc = np.linalg.cholesky(cov)
    s1 = mcmc.hmc_stage1(vg_bad, Lc, eps=0.4, n_leap=6)
    r = mcmc.delayed(f, None, np.tile(mean, (32, 1)), 1500, Lc, n_sub=1, seed=3, max_error=1e9, stage1=s1)
    x = r["chains"][200:].reshape(-1, mean.size)
    assert np.allclose(x.mean(0), mean, atol=0.1)
    assert np.allclose(x.std(0), np.sqrt(np.diag(cov)), rtol=0.1)

    def vg_good(th):
        d = th - mean
        return np.einsum("ij,jk,ik->i", d, icov, d), 2.0 * d @ icov
    s2 = mcmc.hmc_stage1(vg_good, Lc, eps=0.4, n_leap=6)
    d = mcmc.delayed(f, None, np.tile(mean, (32, 1)), 600, Lc, n_sub=1, seed=4, stage1=s2)
    p = mcmc.plain(f, np.tile(mean, (32, 1)), 600, mcmc.proposal_chol(cov), seed=5)
    assert d["stage2_accept"] > 0.99
    assert mcmc.ess(d["chains"], burn=60).min() > 5 * mcmc.ess(p["chains"], burn=60).min()


def test_hmc_stage1_with_a_different_gradient_guide_is_exact():
    """Leapfrog steps driven by another function's gradient (here a wrong,
    smoother one), with the acceptance on the surrogate's own values: the
    transition stays reversible with respect to the surrogate, and after the
    stage-2 correction the chain samples the exact target."""
    mean, cov, icov, f = _target()
    shift = 0.2 * np.sqrt(np.diag(cov))
    icov_s = np.linalg.inv(1.2 * cov)

    def vg_sur(th):
        d = th - mean - shift
        return np.einsum("ij,jk,ik->i", d, icov_s, d), 2.0 * d @ icov_s

    icov_g = np.linalg.inv(np.diag(np.diag(cov)) * 1.5)  # uncorrelated, too wide: a poor guide

    def vg_guide(th):
        d = th - mean
        return np.einsum("ij,jk,ik->i", d, icov_g, d), 2.0 * d @ icov_g

    Lc = np.linalg.cholesky(cov)
    s1 = mcmc.hmc_stage1(vg_sur, Lc, eps=0.4, n_leap=6, guide=vg_guide)
    r = mcmc.delayed(f, None, np.tile(mean, (32, 1)), 1500, Lc, n_sub=1, seed=7, max_error=1e9, stage1=s1)
    x = r["chains"][200:].reshape(-1, mean.size)
    assert np.allclose(x.mean(0), mean, atol=0.1)
    assert np.allclose(x.std(0), np.sqrt(np.diag(cov)), rtol=0.1)
    assert r["accept"] > 0.05


def test_adaptive_pilot_learns_the_covariance_and_the_scale():
    """Started from a proposal 10x too wide and uncorrelated, the pilot's
    pooled covariance approaches the target's and its acceptance moves to
    the 0.234 target."""
    mean, cov, icov, f = _target(P=5, seed=3)
    th0 = np.tile(mean, (32, 1)) + np.random.default_rng(4).normal(0, 0.1, (32, 5))
    r = mcmc.adapt(f, th0, 10.0 * np.eye(5), cycles=6, steps=300, seed=5)
    assert r["accept"][0] < 0.1
    assert 0.15 < r["accept"][-1] < 0.35
    np.testing.assert_allclose(np.sqrt(np.diag(r["cov"])), np.sqrt(np.diag(cov)), rtol=0.25)
    corr = r["cov"] / np.sqrt(np.outer(np.diag(r["cov"]), np.diag(r["cov"])))
    corr_t = cov / np.sqrt(np.outer(np.diag(cov), np.diag(cov)))
    assert np.max(np.abs(corr - corr_t)) < 0.2
