"""Random-walk Metropolis over batched chains, plain and delayed-acceptance.

All log-densities here are GUNDAM's "-2 log L" convention: ``f(theta)`` =
statistical likelihood + prior penalty, and a Metropolis step accepts with
probability min(1, exp(-(f' - f) / 2)) -- the reference's SimpleMcmc uses
-1/2 of its evalFit value as the log-likelihood (SimpleMcmc.cpp:1099-1116)
with the TSimpleMCMC accept rule log U < delta log L (TSimpleMCMC.H:441-460).

* ``plain``: every chain proposes theta' = theta + L z each step and every
  proposal is evaluated by the exact engine (one batched evaluation of all
  chains per step).
* ``delayed``: stage 1 runs, per chain, ``n_sub`` Metropolis steps of the
  same random walk on the surrogate density f_s.  That sub-chain is reversible
  with respect to exp(-f_s/2), so using its end point phi as the proposal, the
  exact Metropolis-Hastings ratio is (Christen & Fox 2005)
      alpha = min(1, exp(-(f(phi) - f(theta))/2 + (f_s(phi) - f_s(theta))/2)),
  which keeps exp(-f/2) exactly invariant however good the surrogate is.
  Chains whose sub-chain did not move skip the exact evaluation.  When the
  running mean of |(f(phi)-f(theta)) - (f_s(phi)-f_s(theta))| exceeds
  ``max_error`` the sampler falls back to plain steps.
"""
from __future__ import annotations

import time

import numpy as np


def proposal_chol(prior_cov, scale=None):
    P = prior_cov.shape[0]
    s = (2.38 ** 2 / P) if scale is None else scale
    return np.linalg.cholesky(s * prior_cov)


def _mh_accept(rng, f_new, f_old):
    u = rng.random(f_new.shape[0])
    with np.errstate(over="ignore", invalid="ignore"):
        return np.log(np.maximum(u, 1e-300)) < -(f_new - f_old) / 2.0


def plain(f_exact, theta0, n_steps, L, seed=0, record=True, thin=1):
    """record: keep every ``thin``-th state ([n_steps // thin x chains x params])."""
    rng = np.random.default_rng(seed)
    th = np.array(theta0, dtype=np.float64)
    C, P = th.shape
    f = f_exact(th)
    out = np.empty((n_steps // thin, C, P)) if record else None
    acc = 0
    n_exact = C
    t0 = time.perf_counter()
    for s in range(n_steps):
        prop = th + rng.standard_normal((C, P)) @ L.T
        fp = f_exact(prop)
        n_exact += C
        a = _mh_accept(rng, fp, f)
        th[a] = prop[a]
        f[a] = fp[a]
        acc += int(a.sum())
        if record and (s + 1) % thin == 0 and (s + 1) // thin <= out.shape[0]:
            out[(s + 1) // thin - 1] = th
    dt = time.perf_counter() - t0
    return {"chains": out, "accept": acc / (n_steps * C), "n_exact": n_exact, "seconds": dt, "final": th}


def adapt(f_exact, theta0, cov0, cycles=4, steps=150, seed=0, target=0.234, record_last=True):
    """Adaptive pilot of the plain sampler, as SimpleMcmc's adaptive proposal
    (covarianceWindow / adaptiveCovTrials, SimpleMcmc.cpp:136-245): cycles of
    ``steps`` random-walk steps; after each cycle the proposal covariance
    becomes the covariance of the second half of the cycle's states pooled
    over all chains, and its scale (starting at 2.38^2/P) moves towards the
    target acceptance.  Returns the final states, the covariance, the scale
    and the acceptance per cycle (and the last cycle's states)."""
    th = np.array(theta0, dtype=np.float64)
    C, P = th.shape
    cov = np.array(cov0, dtype=np.float64)
    scale = 2.38 ** 2 / P
    acc = []
    last = None
    for c in range(cycles):
        L = np.linalg.cholesky(scale * cov + 1e-12 * np.eye(P))
        r = plain(f_exact, th, steps, L, seed=seed + 1000 * c)
        th = r["chains"][-1].copy()
        x = r["chains"][steps // 2:].reshape(-1, P)
        cov = np.cov(x.T) + 1e-12 * np.eye(P)
        acc.append(r["accept"])
        scale *= float(np.exp(2.0 * (r["accept"] - target)))
        last = r["chains"]
    return {"theta": th, "cov": cov, "scale": scale, "accept": acc,
            "chains": last if record_last else None}


def hmc_stage1(value_grad, L, eps=0.25, n_leap=10, n_trans=1, guide=None):
    """Stage 1 of delayed acceptance as Hamiltonian Monte Carlo on the
    surrogate density exp(-f_s/2): returns a callable (theta, fs, n, seed) ->
    (phi, f_s(phi), accepted) for ``delayed(stage1=...)``.

    value_grad(theta [C x P]) -> (f_s [C], d f_s/d theta [C x P]).  Each of the
    ``n_trans`` transitions draws momenta q ~ N(0, I), runs ``n_leap`` leapfrog
    steps of U = f_s/2 with the mass matrix (L L^T)^-1 (x moves by eps L q, q by
    eps L^T grad U), the step jittered per chain uniformly in [0.8, 1.2] x eps
    independently of the state, and accepts with exp(H0 - H1).  Leapfrog with
    any deterministic gradient field is a volume-preserving reversible map, so
    each transition is reversible with respect to exp(-f_s/2) and the
    delayed-acceptance correction keeps the exact posterior invariant.  The
    ``n`` argument of the callable is ignored in favour of ``n_trans`` except
    that n == 0 only evaluates f_s.

    guide: another value_grad whose gradient drives the leapfrog steps (the
    values at the trajectory's ends, and so the acceptance, stay f_s's).  A
    smooth guide (the surrogate's additive base) keeps the trajectories from
    following the network's rounding-level gradient noise; the map is still
    volume-preserving and reversible, so the transition stays reversible with
    respect to exp(-f_s/2)."""
    L = np.asarray(L, dtype=np.float64)
    grad_of = guide if guide is not None else value_grad

    def stage1(theta, fs, n, seed):
        x = np.array(theta, dtype=np.float64)
        C, P = x.shape
        f, g = value_grad(x)
        if guide is not None:
            g = grad_of(x)[1]
        if n == 0:
            return x, f, np.zeros(C, np.int32)
        rng = np.random.default_rng(seed)
        acc = np.zeros(C, np.int32)
        for _ in range(n_trans):
            q = rng.standard_normal((C, P))
            e = eps * rng.uniform(0.8, 1.2, size=(C, 1))
            u = rng.random(C)
            h0 = 0.5 * f + 0.5 * np.sum(q * q, axis=1)
            xn = x.copy()
            qn = q - 0.5 * e * (0.5 * g) @ L
            fn, gn = f, g
            for step in range(n_leap):
                xn = xn + e * (qn @ L.T)
                fn, gn = grad_of(xn)
                if step + 1 < n_leap:
                    qn = qn - e * (0.5 * gn) @ L
            qn = qn - 0.5 * e * (0.5 * gn) @ L
            if guide is not None:
                fn = value_grad(xn)[0]
            h1 = 0.5 * fn + 0.5 * np.sum(qn * qn, axis=1)
            with np.errstate(over="ignore", invalid="ignore"):
                a = np.log(np.maximum(u, 1e-300)) < (h0 - h1)
            x[a], f[a], g[a] = xn[a], fn[a], gn[a]
            acc += a
        return x, f, acc
    return stage1


def delayed(f_exact, f_sur, theta0, n_steps, L, n_sub=10, seed=0, max_error=20.0, record=True, stage1=None,
            thin=1, start_plain=False):
    """stage1: optional callable (theta, fs, n_sub, seed) -> (phi, fphi, n_acc)
    that runs the surrogate sub-chains elsewhere (on the device, with the
    same proposal L and its own random numbers); fs None asks for the
    surrogate values at theta.  Without it the sub-chains run here on f_sur.
    The run falls back to plain steps for good once the running mean of the
    stage-2 error |df - df_s| exceeds max_error (inf: never); start_plain
    runs plain steps from the first one (a fall-back decided elsewhere)."""
    rng = np.random.default_rng(seed)
    th = np.array(theta0, dtype=np.float64)
    C, P = th.shape
    f = f_exact(th)
    if start_plain:
        fs = np.full(C, np.nan)
    else:
        fs = stage1(th, None, 0, seed)[1] if stage1 else f_sur(th)
    out = np.empty((n_steps // thin, C, P)) if record else None

    def keep(s):
        if record and (s + 1) % thin == 0 and (s + 1) // thin <= out.shape[0]:
            out[(s + 1) // thin - 1] = th
    stage1_moves = stage2_tries = stage2_acc = 0
    n_exact = C
    n_sur = C
    err_hist = []
    fell_back_at = 0 if start_plain else None
    t0 = time.perf_counter()
    for s in range(n_steps):
        if fell_back_at is not None:
            prop = th + rng.standard_normal((C, P)) @ L.T
            fp = f_exact(prop)
            n_exact += C
            a = _mh_accept(rng, fp, f)
            th[a] = prop[a]
            f[a] = fp[a]
            fs[a] = np.nan
            stage2_tries += C
            stage2_acc += int(a.sum())
            keep(s)
            continue
        # stage 1: surrogate sub-chain of n_sub random-walk Metropolis steps
        if stage1:
            phi, fphi, _ = stage1(th, fs, n_sub, seed * 1000003 + s + 1)
            n_sur += C * n_sub
        else:
            phi = th.copy()
            fphi = fs.copy()
            for _ in range(n_sub):
                prop = phi + rng.standard_normal((C, P)) @ L.T
                fprop = f_sur(prop)
                n_sur += C
                a = _mh_accept(rng, fprop, fphi)
                phi[a] = prop[a]
                fphi[a] = fprop[a]
        moved = np.any(phi != th, axis=1)
        stage1_moves += int(moved.sum())
        if moved.any():
            idx = np.nonzero(moved)[0]
            fe = f_exact(phi[idx])
            n_exact += idx.size
            stage2_tries += idx.size
            d_exact = fe - f[idx]
            d_sur = fphi[idx] - fs[idx]
            u = rng.random(idx.size)
            with np.errstate(over="ignore", invalid="ignore"):
                a = np.log(np.maximum(u, 1e-300)) < -(d_exact - d_sur) / 2.0
            acc_idx = idx[a]
            th[acc_idx] = phi[acc_idx]
            f[acc_idx] = fe[a]
            fs[acc_idx] = fphi[acc_idx]
            stage2_acc += int(a.sum())
            finite = np.isfinite(d_exact - d_sur)
            err_hist.extend(np.abs(d_exact - d_sur)[finite].tolist())
            recent = err_hist[-4 * C:]
            if len(recent) >= C and np.mean(recent) > max_error:
                fell_back_at = s
        keep(s)
    dt = time.perf_counter() - t0
    return {
        "chains": out,
        "stage1_move_rate": stage1_moves / (n_steps * C),
        "stage2_accept": stage2_acc / max(stage2_tries, 1),
        "accept": stage2_acc / (n_steps * C),
        "n_exact": n_exact,
        "n_surrogate": n_sur,
        "seconds": dt,
        "surrogate_error_mean": float(np.mean(err_hist)) if err_hist else None,
        "fell_back_at_step": fell_back_at,
        "final": th,
    }


def ess(chains, burn=0):
    """Effective sample size per parameter of a set of chains [steps x chains
    x params]: the multi-chain estimator of Vehtari, Gelman, Simpson,
    Carpenter & Buerkner (2021, without rank normalisation or splitting).
    Lag-t autocorrelation from the within-chain autocovariances and the
    between-chain variance, rho_t = 1 - (W - mean_c acov_c(t)) / var+, summed
    with Geyer's initial positive (monotone) sequence.  Chains that have not
    mixed (their means disagree) raise var+ and lower the ESS."""
    x = np.asarray(chains[burn:], dtype=np.float64)
    n, C, P = x.shape
    if n < 4:
        return np.full(P, float(n * C))
    mc = x.mean(axis=0)  # [C x P]
    m = 1 << int(np.ceil(np.log2(2 * n)))
    acov = np.zeros((n, P))
    for c in range(C):
        y = x[:, c, :] - mc[c]
        fy = np.fft.rfft(y, m, axis=0)
        acov += np.fft.irfft(fy * np.conj(fy), m, axis=0)[:n] / n
    acov /= C
    W = acov[0] * n / (n - 1)
    Bn = mc.var(axis=0, ddof=1) if C > 1 else np.zeros(P)
    var_plus = (n - 1) / n * W + Bn
    var_plus = np.where(var_plus > 0, var_plus, 1.0)
    rho = 1.0 - (W - acov) / var_plus
    M = (n - 1) // 2
    gam = rho[0:2 * M:2] + rho[1:2 * M:2]
    pos = gam > 0
    stop = np.where(pos.all(axis=0), M, np.argmin(pos, axis=0))
    mono = np.minimum.accumulate(np.where(pos, gam, 0.0), axis=0)
    keep = np.arange(M)[:, None] < stop[None, :]
    tau = -1.0 + 2.0 * np.where(keep, mono, 0.0).sum(axis=0)
    tau = np.maximum(tau, 1.0 / np.log10(max(n * C, 10)))
    return n * C / tau
