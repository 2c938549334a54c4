"""Surrogate delayed-acceptance MCMC against plain-engine MCMC on one GPU.

    python -m gundam_gb300.da_mcmc [--events N] [--train N] [--epochs E]
                                   [--chains C] [--steps S] [--da-steps S]
                                   [--n-sub M] [--region posterior|prior]
                                   [--proposal adapted|prior]

1. Fit: Gauss-Newton minimum of -2 log L and its Laplace covariance, from
   batched engine launches (``fit.laplace``), as GUNDAM fits before sampling;
   then an adaptive pilot of the plain sampler (``mcmc.adapt``) sets the
   proposal covariance and scale, as SimpleMcmc's adaptive proposal does.
2. Training set: ``--train`` parameter draws from the region (the pilot's
   posterior mean and covariance, or the prior, with the covariance inflated
   x1.5), reweighted exactly by the engine (FP32 dials, FP64 sums) on the
   device; targets are log(sum of weights) per bin after an additive base (one
   piecewise-linear function per parameter and bin) fitted by least squares on
   a host-side subset, which also fits the model of sum(w^2).
3. Surrogate: BF16 MLP (P -> 512 -> 512 -> 512 -> B, SiLU) on the residual,
   Adam with a cosine-decayed learning rate, trained by libgw's own loop.
4. Sampling: C chains of random-walk Metropolis from the pilot's final
   states with the pilot's proposal (``--proposal prior``: 2.38^2/P x the
   prior covariance from the fit's draws).  "plain" evaluates every proposal
   exactly; "delayed" runs n_sub surrogate steps per chain on the device
   (``Surrogate.substeps``) per exact stage-2 correction; "delayed_base_only"
   is the same with the network's output set to zero (the base alone), which
   shows what the network adds.
5. Reported: ESS/s (min and median over parameters, multi-chain estimator
   with Geyer's initial positive sequence, ``mcmc.ess``), stage-2 acceptance, the surrogate's likelihood error against the
   exact one, and the delayed sampler's posterior means and widths against the
   plain sampler's, in units of the posterior width and of their Monte Carlo
   standard errors.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import _native as N
from . import fit as fitmod
from . import mcmc
from .engine import Engine
from .surrogate import Surrogate
from .workload import Workload


def penalty(mean, icov, th):
    d = np.atleast_2d(th) - mean
    return np.sum((d @ icov) * d, axis=1)


def _draws(rng, center, chol, n, inflate=1.0):
    return center[None, :] + inflate * rng.standard_normal((n, center.shape[0])) @ chol.T


def _sampler_stats(ch, seconds, burn):
    e = mcmc.ess(ch, burn=burn)
    return e, {"seconds": seconds, "ess_min": float(e.min()), "ess_median": float(np.median(e)),
               "ess_per_s_min": float(e.min() / seconds), "ess_per_s_median": float(np.median(e) / seconds)}


def run(events=0, train=65536, epochs=20, chains=64, steps=1000, n_sub=10, seed=2, config="c2", log=None,
        precision="fp32", region="posterior", proposal="adapted", base_points=32768, nodes=8, batch=2048,
        lr=1e-3, linear=True, max_error=20.0, adapt_cycles=6, adapt_steps=200, da_steps=None, thin=1,
        warm_steps=500, burn_frac=0.1, stage1="hmc", eps=0.25, n_leap=10, base_only_steps=None):
    """Fit, adapt, train, then sample with both samplers from the same states
    (``steps`` plain steps and ``da_steps`` (default: the same) delayed steps;
    the base-only delayed arm, which shows what the network adds, runs
    ``base_only_steps`` (default: ``da_steps``))."""
    log = log or (lambda *_: None)
    t_all = time.perf_counter()
    da_steps = da_steps or steps
    wl = Workload(config, n_events=events, seed=seed)
    llh_type = N.GW_LLH_BARLOW_BEESTON_OA2021 if config in ("c2", "c5") else N.GW_LLH_POISSON
    k = max(64, chains)
    eng = Engine.from_workload(wl, precision=precision, k_max=k, llh_type=llh_type)
    eng.autotune(chains)
    icov = wl.prior_icov
    P, B = wl.n_params, wl.n_bins

    def f_exact(th):
        out = np.empty(th.shape[0])
        for s in range(0, th.shape[0], k):
            out[s:s + k] = eng.eval(th[s:s + k])[2]
        return out

    # 1. fit, then the adaptive pilot (proposal covariance and scale)
    fr = fitmod.laplace(eng, wl.prior_mean, icov, log=log)
    t0 = time.perf_counter()
    rng0 = np.random.default_rng(seed + 5)
    th_start = _draws(rng0, fr["theta"], np.linalg.cholesky(fr["cov"]), chains, 0.3)
    if proposal == "adapted":
        ad = mcmc.adapt(f_exact, th_start, fr["cov"], cycles=adapt_cycles, steps=adapt_steps, seed=seed + 6)
        cov_post, scale = ad["cov"], ad["scale"]
        th0 = ad["theta"]
        post_samples = ad["chains"][adapt_steps // 2:].reshape(-1, P)
        center = post_samples.mean(axis=0)
    else:
        cov_post, scale = wl.prior_cov, 2.38 ** 2 / P
        th0 = th_start
        post_samples = None
        center = fr["theta"]
    t_adapt = time.perf_counter() - t0
    log(f"pilot: {t_adapt:.2f} s, acceptance {ad['accept'] if proposal == 'adapted' else None}")
    L = np.linalg.cholesky(scale * cov_post)

    # 2. training set: base on a host-side pilot subset, then the device set
    rng = np.random.default_rng(seed + 10)
    if region == "posterior":
        chol_r = np.linalg.cholesky(cov_post)
    else:
        center, chol_r = wl.prior_mean, np.linalg.cholesky(wl.prior_cov)
    t0 = time.perf_counter()
    n_b = min(base_points, train)
    th_b = _draws(rng, center, chol_r, n_b, 1.5)
    sums = np.empty((n_b, B))
    lratio = np.empty((n_b, B))
    for s in range(0, n_b, k):
        a, b, _, _ = eng.eval(th_b[s:s + k])
        sums[s:s + k] = a
        lratio[s:s + k] = np.log(np.maximum(b, 1e-300)) - np.log(np.maximum(a, 1e-300))
    t_base_data = time.perf_counter() - t0
    sur = Surrogate(P, B, batch_max=4096, seed=seed)
    t1 = time.perf_counter()
    sur.fit_additive(th_b, np.log(np.maximum(sums, 1e-300)), log_ratio=lratio, nodes=nodes)
    t_base_fit = time.perf_counter() - t1
    del lratio
    sur.attach(wl.data, None, llh_type)
    sur.reserve(train)
    sur.append(th_b, sums)
    del sums
    left = train - n_b
    while left > 0:
        m = min(65536, left)
        sur.append_eval(eng, _draws(rng, center, chol_r, m, 1.5), k=k)
        left -= m
    t_data = time.perf_counter() - t0
    log(f"training set: {train} points in {t_data:.2f} s (base fit {t_base_fit:.2f} s)")

    # 3. training
    t0 = time.perf_counter()
    hist = sur.train(epochs=epochs, lr=lr, batch=min(batch, train - train % 8))
    t_train = time.perf_counter() - t0
    log(f"training: {epochs} epochs, {t_train:.2f} s, loss {hist[0]:.4g} -> {hist[-1]:.4g}")

    def make_f_sur(su):
        return lambda th: su.stat_llh(th) + penalty(wl.prior_mean, icov, th)

    f_sur = make_f_sur(sur)
    sur.set_chain(L, wl.prior_mean, icov)
    lin = None
    if linear:
        lin = sur.linear_twin()
        lin.attach(wl.data, None, llh_type)
        lin.set_chain(L, wl.prior_mean, icov)

    # surrogate error: sd of the differences between points at posterior
    # states, and of the change over n_sub-step random-walk excursions
    hrng = np.random.default_rng(seed + 99)
    if post_samples is not None:
        test = post_samples[hrng.choice(post_samples.shape[0], 256, replace=False)]
    else:
        test = _draws(hrng, center, chol_r, 256)
    excur = test + (hrng.standard_normal((256, n_sub, P)) @ L.T).sum(axis=1)
    f_t, f_e = f_exact(test), f_exact(excur)

    def errs(su):
        fs = make_f_sur(su)
        e1 = fs(test) - f_t
        e2 = fs(excur) - f_e
        return {"posterior": float(np.std(e1 - e1.mean())), "excursion_difference": float(np.std(e2 - e1))}
    err = {"with_network": errs(sur)}
    if lin:
        err["base_only"] = errs(lin)
    err["exact_excursion_spread"] = float(np.std(f_e - f_t))
    t0 = time.perf_counter()
    for r in range(5):
        sur.substeps(th0, None, n_sub, r)
    t_sub = (time.perf_counter() - t0) / 5
    t0 = time.perf_counter()
    for r in range(5):
        sur.value_grad(th0)
    t_grad = (time.perf_counter() - t0) / 5
    t0 = time.perf_counter()
    for _ in range(5):
        f_exact(th0)
    t_exact = (time.perf_counter() - t0) / 5

    # 4. sampling, both samplers from the same states with the same proposal
    L_post = np.linalg.cholesky(cov_post)

    def stage1_of(su):
        if stage1 == "hmc":
            return mcmc.hmc_stage1(su.value_grad, L_post, eps=eps, n_leap=n_leap)
        if stage1 == "hmc_base_grad":  # leapfrog on the base's gradient, acceptance on the full surrogate
            return mcmc.hmc_stage1(su.value_grad, L_post, eps=eps, n_leap=n_leap,
                                   guide=lin.value_grad if lin is not None and su is not lin else None)
        return lambda th, fs, ns, sd: su.substeps(th, fs, ns, sd)
    # both samplers start from the same states, taken after a delayed-
    # acceptance warm-up (it mixes fastest) so that neither starts out of
    # equilibrium; the first burn_frac of each run is discarded as well
    # The fall-back to plain steps is decided in the warm-up alone and frozen
    # for the recorded run: a switch that depends on the recorded chain's own
    # history would make the recorded sampler adaptive.  A warm-up that fell
    # back makes the recorded delayed-acceptance arm plain from its first step.
    t0 = time.perf_counter()
    warm_fell_back = None
    if warm_steps > 0:
        w = mcmc.delayed(f_exact, f_sur, th0, warm_steps, L, n_sub=n_sub, seed=seed + 3, max_error=max_error,
                         stage1=stage1_of(sur), record=False)
        th0 = w["final"]
        warm_fell_back = w["fell_back_at_step"]
    t_warm = time.perf_counter() - t0
    frozen = dict(max_error=float("inf"), start_plain=warm_fell_back is not None)
    p = mcmc.plain(f_exact, th0, steps, L, seed=seed + 7, thin=thin)
    d = mcmc.delayed(f_exact, f_sur, th0, da_steps, L, n_sub=n_sub, seed=seed + 8, stage1=stage1_of(sur),
                     thin=thin, **frozen)
    dl = mcmc.delayed(f_exact, None, th0, base_only_steps or da_steps, L, n_sub=n_sub, seed=seed + 9,
                      max_error=float("inf"), stage1=stage1_of(lin), thin=thin) if lin else None
    bp = int(burn_frac * p["chains"].shape[0])
    bd = int(burn_frac * d["chains"].shape[0])
    ess_p, st_p = _sampler_stats(p["chains"], p["seconds"], bp)
    ess_d, st_d = _sampler_stats(d["chains"], d["seconds"], bd)
    xp = p["chains"][bp:].reshape(-1, P)
    xd = d["chains"][bd:].reshape(-1, P)
    sig_p, sig_d = xp.std(0), xd.std(0)
    mean_diff = np.abs(xd.mean(0) - xp.mean(0))
    se = np.sqrt(sig_p ** 2 / ess_p + sig_d ** 2 / ess_d)
    worst_d = np.argsort(ess_d)[:8]
    worst_p = np.argsort(ess_p)[:8]
    res = {
        "slowest_parameters": {"delayed": [[int(i), float(ess_d[i]), float(ess_p[i])] for i in worst_d],
                               "plain": [[int(i), float(ess_p[i]), float(ess_d[i])] for i in worst_p],
                               "columns": "parameter, ESS of this sampler, ESS of the other"},
        "workload": f"{config}: {wl.n_events} events, {wl.n_dials} dials, {B} bins, {P} params",
        "precision": precision, "chains": chains, "plain_steps": steps, "delayed_steps": da_steps, "n_sub": n_sub,
        "thin": thin, "warm_steps": warm_steps, "warm_seconds": t_warm, "burn_fraction": burn_frac,
        "fallback": {"decided_in": "warm-up", "warm_up_fell_back_at_step": warm_fell_back,
                     "recorded_run_plain_from_start": warm_fell_back is not None},
        "fit": {"f": fr["f"], "iterations": fr["iterations"], "seconds": fr["seconds"]},
        "pilot": {"proposal": proposal, "seconds": t_adapt, "scale": scale,
                  "accept": ad["accept"] if proposal == "adapted" else None,
                  "posterior_sd_median": float(np.median(np.sqrt(np.diag(cov_post))))},
        "training": {"region": region, "points": train, "epochs": epochs, "base": f"additive, {nodes} nodes",
                     "base_points": n_b, "base_data_seconds": t_base_data, "base_fit_seconds": t_base_fit,
                     "data_seconds": t_data, "train_seconds": t_train, "loss_first_last": [hist[0], hist[-1]]},
        "surrogate_llh_error_sd": err,
        "seconds_per_step": {"surrogate_substeps": t_sub, "surrogate_value_grad": t_grad, "exact": t_exact,
                             "points": chains},
        "stage1": {"kind": stage1, "n_sub": n_sub} if stage1 == "rwm" else
                  {"kind": stage1, "eps": eps, "n_leap": n_leap, "mass": "posterior covariance from the pilot",
                   "leapfrog_gradient": "the additive base's" if stage1 == "hmc_base_grad" else "the surrogate's"},
        "plain": dict(st_p, accept=p["accept"], n_exact=p["n_exact"]),
        "delayed": dict(st_d, stage2_accept=d["stage2_accept"], accept=d["accept"], n_exact=d["n_exact"],
                        n_surrogate=d["n_surrogate"], fell_back_at_step=d["fell_back_at_step"],
                        stage2_llh_error_mean=d["surrogate_error_mean"]),
        "posterior": {
            "mean_diff_over_sigma_max": float((mean_diff / sig_p).max()),
            "mean_diff_over_sigma_median": float(np.median(mean_diff / sig_p)),
            "mean_diff_over_mc_se_max": float((mean_diff / se).max()),
            "mean_diff_over_mc_se_rms": float(np.sqrt(np.mean((mean_diff / se) ** 2))),
            "width_ratio_range": [float((sig_d / sig_p).min()), float((sig_d / sig_p).max())],
            "width_ratio_median": float(np.median(sig_d / sig_p)),
            # resolution: the Monte Carlo standard error of the mean difference
            # in units of sigma, and of the relative width difference (a width
            # estimated from ESS draws has relative error ~ 1 / sqrt(2 ESS))
            "mean_diff_mc_se_over_sigma_median": float(np.median(se / sig_p)),
            "mean_diff_mc_se_over_sigma_max": float((se / sig_p).max()),
            "width_diff_over_sigma_max": float((np.abs(sig_d - sig_p) / sig_p).max()),
            "width_diff_mc_se_median": float(np.median(np.sqrt(0.5 / ess_p + 0.5 / ess_d))),
            "width_diff_over_mc_se_max": float((np.abs(sig_d - sig_p) / sig_p /
                                               np.sqrt(0.5 / ess_p + 0.5 / ess_d)).max()),
        },
        "ess_per_s_gain_min": st_d["ess_per_s_min"] / st_p["ess_per_s_min"],
        "ess_per_s_gain_median": st_d["ess_per_s_median"] / st_p["ess_per_s_median"],
    }
    if dl is not None:
        _, st_l = _sampler_stats(dl["chains"], dl["seconds"], int(burn_frac * dl["chains"].shape[0]))
        res["delayed_base_only"] = dict(st_l, steps=base_only_steps or da_steps, stage2_accept=dl["stage2_accept"],
                                        fell_back_at_step=dl["fell_back_at_step"],
                                        stage2_llh_error_mean=dl["surrogate_error_mean"])
        res["network_gain_ess_per_s_median"] = st_d["ess_per_s_median"] / st_l["ess_per_s_median"]
        lin.close()
    res["total_seconds"] = time.perf_counter() - t_all
    sur.close()
    eng.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--events", type=int, default=0)
    ap.add_argument("--train", type=int, default=65536)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--chains", type=int, default=64)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--da-steps", type=int, default=0)
    ap.add_argument("--n-sub", type=int, default=10)
    ap.add_argument("--nodes", type=int, default=8)
    ap.add_argument("--config", default="c2")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "df64"])
    ap.add_argument("--region", default="posterior", choices=["posterior", "prior"])
    ap.add_argument("--proposal", default="adapted", choices=["adapted", "prior"])
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--thin", type=int, default=1)
    ap.add_argument("--warm-steps", type=int, default=500)
    ap.add_argument("--stage1", default="hmc", choices=["hmc", "hmc_base_grad", "rwm"])
    ap.add_argument("--eps", type=float, default=0.25)
    ap.add_argument("--n-leap", type=int, default=10)
    ap.add_argument("--no-linear", action="store_true")
    ap.add_argument("--base-only-steps", type=int, default=0)
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    lg = (lambda m: print(m, file=sys.stderr, flush=True)) if a.verbose else None
    print(json.dumps(run(a.events, a.train, a.epochs, a.chains, a.steps, a.n_sub, config=a.config,
                         precision=a.precision, region=a.region, proposal=a.proposal, nodes=a.nodes,
                         linear=not a.no_linear, log=lg, da_steps=a.da_steps or None, lr=a.lr, thin=a.thin,
                         warm_steps=a.warm_steps, stage1=a.stage1, eps=a.eps, n_leap=a.n_leap,
                         base_only_steps=a.base_only_steps or None)))


if __name__ == "__main__":
    main()
