"""Best fit and Laplace covariance of f = -2 log L through the batched engine.

GUNDAM fits (MINUIT MIGRAD + HESSE) before it samples, and its MCMC can take
the proposal covariance from that fit (``adaptiveCovFile`` / ``adaptiveCovName``,
src/Fitter/Minimizer/src/SimpleMcmc.cpp:179-196).  The minimiser here is a
Gauss-Newton iteration built on K-point engine launches:

* the Jacobian J [P x B] of the log bin rates by central differences: 2P
  points, evaluated K per launch;
* the gradient of f (statistical LLH + prior penalty, as the engine returns
  it) from the same 2P evaluations;
* H = 2 J diag(v) J^T + 2 C^-1 with v_b = mu_b / (1 + Sum w^2_b / mu_b): the
  Poisson information of bin b in log-rate units (d^2 f / d(log mu)^2 = 2 mu),
  reduced by the Monte Carlo statistical variance that the Barlow-Beeston term
  adds to the prediction; C^-1 is the prior's inverse covariance;
* a line search along the Newton step: one launch over K step lengths.

The covariance of the parameters at the optimum is (H / 2)^-1, f being -2 log L.
"""
from __future__ import annotations

import time

import numpy as np


def _eval_rows(eng, pts, k):
    n = pts.shape[0]
    sums = np.empty((n, eng.n_bins))
    sums2 = np.empty((n, eng.n_bins))
    f = np.empty(n)
    for s in range(0, n, k):
        a, b, c, _ = eng.eval(pts[s:s + k])
        sums[s:s + k], sums2[s:s + k], f[s:s + k] = a, b, c
    return sums, sums2, f


def laplace(eng, prior_mean, prior_icov, theta0=None, h=None, max_iter=10, tol=1e-3, k=None, log=None):
    """Gauss-Newton minimum of the engine's LLH and its Laplace covariance.

    Returns {"theta", "cov", "f", "iterations", "evaluations", "seconds", "history"}."""
    t0 = time.perf_counter()
    P = prior_mean.shape[0]
    k = k or eng.k_max
    th = np.array(prior_mean if theta0 is None else theta0, dtype=np.float64)
    h = np.full(P, 1e-2) if h is None else np.broadcast_to(np.asarray(h, dtype=np.float64), (P,)).copy()
    n_eval = 0
    history = []
    H = None
    f0 = np.nan
    it = 0
    for it in range(1, max_iter + 1):
        E = np.diag(h)
        pts = np.vstack([th[None, :], th + E, th - E])
        sums, sums2, f = _eval_rows(eng, pts, k)
        n_eval += pts.shape[0]
        f0 = f[0]
        mu = sums[0]
        ok = mu > 0
        logs = np.log(np.maximum(sums, 1e-300))
        J = (logs[1:1 + P] - logs[1 + P:]) / (2.0 * h[:, None])
        J[:, ~ok] = 0.0
        g = (f[1:1 + P] - f[1 + P:]) / (2.0 * h)
        v = np.where(ok, mu / (1.0 + sums2[0] / np.maximum(mu, 1e-300)), 0.0)
        H = 2.0 * (J * v) @ J.T + 2.0 * prior_icov
        step = np.linalg.solve(H, g)
        alphas = np.concatenate([[0.0], np.geomspace(1.5, 1e-3, k - 1)])
        cand = th[None, :] - alphas[:, None] * step[None, :]
        _, _, fc = _eval_rows(eng, cand, k)
        n_eval += cand.shape[0]
        best = int(np.nanargmin(fc))
        dec = f0 - fc[best]
        history.append({"f": float(f0), "decrease": float(dec), "alpha": float(alphas[best]),
                        "grad_norm": float(np.linalg.norm(g))})
        if log:
            log(f"fit iteration {it}: f {f0:.6f} -> {fc[best]:.6f} (alpha {alphas[best]:.3g})")
        th = cand[best].copy()
        if dec < tol:
            f0 = float(fc[best])
            break
    cov = 2.0 * np.linalg.inv(H)
    cov = 0.5 * (cov + cov.T)
    return {"theta": th, "cov": cov, "f": float(f0), "iterations": it, "evaluations": n_eval,
            "seconds": time.perf_counter() - t0, "history": history}
