"""Surrogate delayed-acceptance MCMC against plain-engine MCMC on one GPU.

    python -m gundam_gb300.da_mcmc [--events N] [--train N] [--epochs E]
                                   [--chains C] [--steps S] [--n-sub M]

1. Training set: ``--train`` parameter draws from the prior with its
   covariance inflated x1.5, reweighted exactly by the engine (FP32 dials,
   FP64 sums); targets are log(sum of weights) per bin.
2. Surrogate: affine least-squares base + BF16 MLP (P -> 512 -> 512 -> 512 -> B,
   SiLU) on the residual, Adam with a cosine-decayed learning rate.
3. Sampling: C chains of random-walk Metropolis with proposal covariance
   2.38^2/P x prior covariance; "plain" evaluates every proposal exactly,
   "delayed" runs n_sub surrogate steps per exact stage-2 correction.
4. Reported: ESS/s (min and median over parameters, Geyer initial positive
   sequence), stage-2 acceptance, the surrogate's likelihood error against the
   exact one on held-out draws, and the posterior means / widths of the two
   samplers in units of the posterior width.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import _native as N
from . import mcmc
from .engine import Engine
from .surrogate import Surrogate, training_data
from .workload import Workload


def penalty(wl, icov, th):
    d = np.atleast_2d(th) - wl.prior_mean
    return np.einsum("ij,jk,ik->i", d, icov, d)


def run(events=0, train=16384, epochs=20, chains=64, steps=400, n_sub=10, seed=2, config="c2", log=print,
        precision="fp32", region="pilot", pilot_steps=200):
    """region: where the training draws come from -- "prior" (the prior with
    its covariance inflated x1.5) or "pilot" (a short plain-MCMC pilot run:
    its sample mean with its sample covariance inflated x1.5)."""
    t_all = time.perf_counter()
    wl = Workload(config, n_events=events, seed=seed)
    llh_type = N.GW_LLH_BARLOW_BEESTON_OA2021 if config in ("c2", "c5") else N.GW_LLH_POISSON
    eng = Engine.from_workload(wl, precision=precision, k_max=max(64, chains), llh_type=llh_type)
    eng.autotune(chains)
    icov = wl.prior_icov

    def f_exact(th):
        out = np.empty(th.shape[0])
        for s in range(0, th.shape[0], 64):
            out[s:s + 64] = eng.eval(th[s:s + 64])[2]
        return out

    L = mcmc.proposal_chol(wl.prior_cov)
    th0 = wl.draw_points(chains, seed + 5, inflate=0.3)
    # pilot / burn-in with the plain sampler (shared by both samplers below)
    t0 = time.perf_counter()
    pilot = mcmc.plain(f_exact, th0, pilot_steps, L, seed=seed + 6)
    t_pilot = time.perf_counter() - t0
    th0 = pilot["chains"][-1].copy()
    pil = pilot["chains"][pilot_steps // 2:].reshape(-1, wl.n_params)
    t0 = time.perf_counter()
    if region == "prior":
        thetas, logs, ratio = training_data(eng, wl, train, seed=seed + 10, inflate=1.5)
    else:
        mean = pil.mean(0)
        cov = np.cov(pil.T) + 1e-12 * np.eye(wl.n_params)
        rng = np.random.default_rng(seed + 10)
        thetas = mean + 1.5 * rng.standard_normal((train, wl.n_params)) @ np.linalg.cholesky(cov).T
        logs = np.empty((train, wl.n_bins))
        ratio = np.zeros(wl.n_bins)
        for s0 in range(0, train, 64):
            sums, sums2, _, _ = eng.eval(thetas[s0:s0 + 64])
            logs[s0:s0 + 64] = np.log(np.maximum(sums, 1e-300))
            ratio += (sums2 / np.maximum(sums, 1e-300)).sum(axis=0)
        ratio /= train
    t_data = time.perf_counter() - t0
    sur = Surrogate(wl.n_params, wl.n_bins, batch_max=4096, seed=seed)
    t0 = time.perf_counter()
    hist = sur.fit(thetas, logs, epochs=epochs, lr=1e-3, batch=min(2048, train))
    t_train = time.perf_counter() - t0
    sur.attach(wl.data, ratio, llh_type)

    def f_sur(th):
        return sur.stat_llh(th) + penalty(wl, icov, th)

    # surrogate error (sd of the differences between points) on held-out
    # prior draws and on held-out pilot-chain states
    def err_sd(pts):
        ex = f_exact(pts)
        sx = f_sur(pts)
        return float(np.std((ex - ex.mean()) - (sx - sx.mean())))
    sur_err_prior = err_sd(wl.draw_points(256, seed + 99))
    sur_err_post = err_sd(pil[np.random.default_rng(seed + 98).choice(pil.shape[0], 256, replace=False)])

    p = mcmc.plain(f_exact, th0, steps, L, seed=seed + 7)
    d = mcmc.delayed(f_exact, f_sur, th0, steps, L, n_sub=n_sub, seed=seed + 8)
    b = steps // 5
    ess_p = mcmc.ess(p["chains"], burn=b)
    ess_d = mcmc.ess(d["chains"], burn=b)
    xp = p["chains"][b:].reshape(-1, wl.n_params)
    xd = d["chains"][b:].reshape(-1, wl.n_params)
    sig = xp.std(0)
    res = {
        "workload": f"{config}: {wl.n_events} events, {wl.n_dials} dials, {wl.n_bins} bins, {wl.n_params} params",
        "train_points": train, "epochs": epochs, "train_seconds": t_train, "data_seconds": t_data,
        "train_mse_first_last": [hist[0], hist[-1]],
        "training_region": region, "pilot_steps": pilot_steps, "pilot_seconds": t_pilot,
        "surrogate_llh_error_sd_prior_draws": sur_err_prior,
        "surrogate_llh_error_sd_posterior": sur_err_post,
        "chains": chains, "steps": steps, "n_sub": n_sub,
        "plain": {"seconds": p["seconds"], "accept": p["accept"], "n_exact": p["n_exact"],
                  "ess_min": float(ess_p.min()), "ess_median": float(np.median(ess_p)),
                  "ess_per_s_min": float(ess_p.min() / p["seconds"]),
                  "ess_per_s_median": float(np.median(ess_p) / p["seconds"])},
        "delayed": {"seconds": d["seconds"], "stage2_accept": d["stage2_accept"], "accept": d["accept"],
                    "n_exact": d["n_exact"], "n_surrogate": d["n_surrogate"],
                    "fell_back_at_step": d["fell_back_at_step"],
                    "stage2_llh_error_mean": d["surrogate_error_mean"],
                    "ess_min": float(ess_d.min()), "ess_median": float(np.median(ess_d)),
                    "ess_per_s_min": float(ess_d.min() / d["seconds"]),
                    "ess_per_s_median": float(np.median(ess_d) / d["seconds"])},
        "posterior_mean_diff_over_sigma_max": float(np.max(np.abs(xp.mean(0) - xd.mean(0)) / sig)),
        "posterior_width_ratio_range": [float(np.min(xd.std(0) / sig)), float(np.max(xd.std(0) / sig))],
        "total_seconds": time.perf_counter() - t_all,
    }
    res["ess_per_s_gain_min"] = res["delayed"]["ess_per_s_min"] / max(res["plain"]["ess_per_s_min"], 1e-300)
    res["ess_per_s_gain_median"] = res["delayed"]["ess_per_s_median"] / max(res["plain"]["ess_per_s_median"], 1e-300)
    sur.close()
    eng.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--events", type=int, default=0)
    ap.add_argument("--train", type=int, default=16384)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--chains", type=int, default=64)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--n-sub", type=int, default=10)
    ap.add_argument("--config", default="c2")
    ap.add_argument("--region", default="pilot", choices=["pilot", "prior"])
    ap.add_argument("--pilot-steps", type=int, default=200)
    a = ap.parse_args()
    print(json.dumps(run(a.events, a.train, a.epochs, a.chains, a.steps, a.n_sub, config=a.config,
                         region=a.region, pilot_steps=a.pilot_steps)))


if __name__ == "__main__":
    main()
