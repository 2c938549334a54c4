"""The Gauss-Newton fit (gundam_gb300/fit.py) on the CPU, through a stand-in
engine whose bin rates are exp(c + W theta) with Poisson data and a Gaussian
prior: the minimum agrees with a general-purpose minimiser and the Laplace
covariance with the inverse Hessian of -log L."""
import numpy as np
import pytest

from gundam_gb300.fit import laplace

scipy_optimize = pytest.importorskip("scipy.optimize")


class ToyEngine:
    """eval(points) -> (sum w, sum w^2, LLH, statistical LLH) like Engine.eval."""

    def __init__(self, seed=0, P=3, B=40):
        rng = np.random.default_rng(seed)
        self.n_bins, self.k_max = B, 16
        self.c = rng.uniform(2.0, 5.0, B)
        self.W = rng.normal(0.0, 0.3, (B, P))
        self.theta_true = rng.normal(0.0, 0.5, P)
        self.data = rng.poisson(np.exp(self.c + self.W @ self.theta_true)).astype(np.float64)
        self.icov = 0.5 * np.eye(P)

    def f(self, th):
        mu = np.exp(self.c + self.W @ th)
        n = self.data
        with np.errstate(divide="ignore", invalid="ignore"):
            t = np.where(n > 0, n * np.log(n / mu), 0.0)
        stat = float(np.sum(2.0 * (mu - n + t)))
        return stat + float(th @ self.icov @ th), stat

    def eval(self, pts):
        pts = np.atleast_2d(pts)
        mu = np.exp(self.c[None, :] + pts @ self.W.T)
        fs = np.array([self.f(p) for p in pts])
        return mu, np.zeros_like(mu), fs[:, 0], fs[:, 1]


def test_gauss_newton_minimum_and_laplace_covariance():
    eng = ToyEngine()
    P = eng.W.shape[1]
    r = laplace(eng, np.zeros(P), eng.icov, max_iter=20, tol=1e-9)
    ref = scipy_optimize.minimize(lambda t: eng.f(t)[0], np.zeros(P), method="BFGS", options={"gtol": 1e-10})
    np.testing.assert_allclose(r["theta"], ref.x, atol=1e-4)
    assert r["f"] <= ref.fun + 1e-6
    # -log L = f / 2: covariance = inverse Hessian of f / 2, by central differences
    h = 1e-4
    H = np.empty((P, P))
    for i in range(P):
        for j in range(P):
            e_i, e_j = np.eye(P)[i] * h, np.eye(P)[j] * h
            H[i, j] = (eng.f(ref.x + e_i + e_j)[0] - eng.f(ref.x + e_i - e_j)[0]
                       - eng.f(ref.x - e_i + e_j)[0] + eng.f(ref.x - e_i - e_j)[0]) / (4 * h * h)
    cov = np.linalg.inv(H / 2.0)
    np.testing.assert_allclose(r["cov"], cov, rtol=0.1, atol=1e-4)
    assert r["evaluations"] > 0 and r["iterations"] >= 1
