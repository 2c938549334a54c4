#!/usr/bin/env python
"""Benchmark of the reweighting path: LLH evaluations per second.

Default workload: the 5M-event mixed-dial configuration (8 samples, 3000
bins, 200 correlated parameters, Barlow-Beeston likelihood), dial math and
weight products in FP32 with bin sums / sum of w^2 / likelihood in FP64,
K = 64 parameter points per pass.  One step is one pass over all events for
the K points.  The dial payload (~2.7 GB) is larger than L2, so no flush is
needed between steps.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Under torchrun each rank evaluates its own replica (the path shards by
events; this build runs replicas only) and rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "LLH evals/s (5M events, C2 mixed dials)"
# the K = 1 kernels by gw_get_plain_kernel value
PLAIN_NAMES = ["k_plain", "k_plain_ws", "k_plain_ws (8 evaluator warps)"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gw", choices=["gw", "reference"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--events", type=int, default=0)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--points", type=int, default=64)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-mcmc", action="store_true")
    ap.add_argument("--no-c5", action="store_true")
    ap.add_argument("--mcmc-steps", type=int, default=20000)
    ap.add_argument("--mcmc-base-only-steps", type=int, default=4000)
    ap.add_argument("--mcmc-train", type=int, default=1 << 20)
    ap.add_argument("--mcmc-epochs", type=int, default=20)
    ap.add_argument("--mcmc-nsub", type=int, default=40)
    ap.add_argument("--mcmc-stage1", default="hmc", choices=["hmc", "rwm"])
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if args.impl == "gw" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def max_over_ranks(x: float, dist, device="cuda") -> float:
    """Largest value over all ranks (the slowest rank's time)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units all ranks processed divided by the (max-over-ranks) time."""
    return world * units_per_rank / seconds


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def llh_type_for(cfg):
    from gundam_gb300 import _native as N

    return N.GW_LLH_BARLOW_BEESTON_OA2021 if cfg in ("c2", "c5") else N.GW_LLH_POISSON


def cpu_baseline(wl, cfg, seconds, threads=None):
    """The CPU propagation (oracle port) timed on this host: full evaluations, K=1."""
    from oracle.oracle import Oracle

    threads = threads or (os.cpu_count() or 1)
    orc = Oracle(wl, llh_type=llh_type_for(cfg))
    p = wl.nominal()
    orc.eval(p, threads=threads)  # warm caches
    t0 = time.perf_counter()
    orc.eval(p, threads=threads)
    one = time.perf_counter() - t0
    n = max(1, min(200, int(seconds / max(one, 1e-6))))
    pts = wl.draw_points(n, 4242)
    t0 = time.perf_counter()
    for i in range(n):
        orc.eval(pts[i:i + 1], threads=threads)
    dt = time.perf_counter() - t0
    orc.close()
    return n / dt, threads, n, dt


def run_reference(args, world, rank, dist):
    if rank != 0:
        return
    from gundam_gb300 import Workload

    wl = Workload(args.config, n_events=args.events, seed=args.seed)
    from oracle.oracle import Oracle

    threads = os.cpu_count() or 1
    orc = Oracle(wl, llh_type=llh_type_for(args.config))
    pts = wl.draw_points(args.warmup + args.steps, 77)
    for i in range(args.warmup):
        orc.eval(pts[i:i + 1], threads=threads)
    t0 = time.perf_counter()
    for i in range(args.steps):
        orc.eval(pts[args.warmup + i:args.warmup + i + 1], threads=threads)
    dt = time.perf_counter() - t0
    v = args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.config}: {wl.n_events} events, {wl.n_dials} dials, {wl.n_bins} bins, "
                               f"{wl.n_params} params", "points_per_step": 1, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": v, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full evaluations of all {wl.n_events} events"},
        "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_device(eng, torch, d, K, steps, warmup, dist):
    # a dedicated stream: the legacy default stream has handle 0, which the
    # C ABI reads as "the engine's own stream"
    stream = d.setdefault("stream", torch.cuda.Stream())
    sp = stream.cuda_stream
    for _ in range(warmup):
        eng.eval_device(d["p"].data_ptr(), K, d["s"].data_ptr(), d["s2"].data_ptr(), d["l"].data_ptr(), 0, sp)
    torch.cuda.synchronize()
    eng.sync()
    eng.set_profiling(True)
    eng.read_profile()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        eng.eval_device(d["p"].data_ptr(), K, d["s"].data_ptr(), d["s2"].data_ptr(), d["l"].data_ptr(), 0, sp)
    b.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = a.elapsed_time(b) / steps
    kms, klaunch, launches = eng.read_profile()
    eng.set_profiling(False)
    eng.sync()
    return ms, kms / max(1, klaunch), launches


def cpu_baseline_checks(c1_check, c3_check, c5_check, threads=None):
    """The CPU-baseline leg's second task: the CPU propagation (FP64) of the
    same parameter points the engine evaluated for C1, C3 and C5, timed, and
    the engine's per-bin and LLH errors against it."""
    from gundam_gb300 import Workload
    from oracle.oracle import Oracle

    threads = threads or (os.cpu_count() or 1)
    res = {}
    if c1_check is not None or c3_check is not None:
        wl = Workload("c1", seed=2)
        orc = Oracle(wl, llh_type=llh_type_for("c1"))
        if c1_check is not None:
            t0 = time.perf_counter()
            ref = orc.eval(c1_check["points"], threads=threads)
            dt = time.perf_counter() - t0
            res["c1"] = {"cpu_evals_per_s": len(c1_check["points"]) / dt, "cpu_threads": threads}
            for key, (sums, llh) in c1_check["outputs"].items():
                res["c1"][key] = errors_vs_oracle(sums, llh, ref)
        if c3_check is not None:
            res["c3"] = {}
            for key, pts in c3_check["points"].items():
                sums, llh = c3_check["outputs"][key]
                res["c3"][key] = errors_vs_oracle(sums, llh, orc.eval(pts, threads=threads))
        orc.close()
        wl.close()
    if c5_check is not None:
        from gundam_gb300.stress import host_available_gb

        need = 1.6 * c5_check["events"] / 1e6  # GB: the workload (~60 GB at 40M events) and the CPU path's arrays
        if host_available_gb() < need:
            res["c5"] = {"skipped": f"host has {host_available_gb():.0f} GB available, the check needs ~{need:.0f} GB"}
            return res
        # the 40M-event workload again (the GPU run released its copy)
        wl = Workload("c5", n_events=c5_check["events"], seed=c5_check["seed"])
        orc = Oracle(wl, llh_type=llh_type_for("c5"))
        t0 = time.perf_counter()
        ref = orc.eval(c5_check["points"], threads=threads)
        dt = time.perf_counter() - t0
        res["c5"] = {"cpu_evals_per_s": len(c5_check["points"]) / dt, "cpu_threads": threads,
                     "points": len(c5_check["points"])}
        for key, (sums, llh) in c5_check["outputs"].items():
            k = len(llh)
            res["c5"][key] = errors_vs_oracle(sums, llh, {"sums": ref["sums"][:k], "llh": ref["llh"][:k]})
        orc.close()
        wl.close()
    return res


def errors_vs_oracle(sums, llh, ref):
    """Largest per-bin relative error of the bin sums (bins the oracle leaves
    empty must be 0 exactly) and largest absolute LLH error."""
    import numpy as np

    r = ref["sums"]
    occ = r != 0
    rel = np.abs(sums[occ] - r[occ]) / np.abs(r[occ])
    return {"max_bin_rel_err": float(rel.max(initial=0.0)),
            "empty_bins_exact": bool(np.all(sums[~occ] == 0.0)),
            "max_llh_abs_err": float(np.max(np.abs(llh - ref["llh"])))}


def c1_points(local, n_points=1000):
    """C1 (100k events, Poisson LLH, 20 parameters): bin contents and LLH at
    1000 random parameter points from the prior, FP64 engine (the plain K = 1
    kernel point by point, and all 1000 in batched launches of 250) and FP32
    dials; rates through gw_eval with host buffers.  Returns the record and
    the engine outputs, which the CPU-baseline leg checks against the CPU
    propagation of the same points."""
    import numpy as np

    from gundam_gb300 import Engine, Workload

    wl = Workload("c1", seed=2)
    pts = wl.draw_points(n_points, 2024)
    out = {"workload": f"c1: {wl.n_events} events, {wl.n_dials} dials, {wl.n_bins} bins, {wl.n_params} params",
           "points": n_points,
           "tolerance": {"fp64": "per-bin relative 1e-12, LLH absolute 1e-6",
                         "fp32": "per-bin relative 2e-5, LLH absolute 5e-2"}}
    outputs = {}
    for prec, K in (("fp64", 1), ("fp64", 250), ("fp32", 250)):
        eng = Engine.from_workload(wl, precision=prec, k_max=K, llh_type=llh_type_for("c1"), device=local)
        eng.autotune(K)
        sums = np.empty((n_points, wl.n_bins))
        llh = np.empty(n_points)
        eng.eval(pts[:K])
        t0 = time.perf_counter()
        for a in range(0, n_points, K):
            s_, _, l_, _ = eng.eval(pts[a:a + K])
            sums[a:a + K], llh[a:a + K] = s_, l_
        dt = time.perf_counter() - t0
        out[f"{prec}_K{K}"] = {"evals_per_s": n_points / dt, "launches_of_points": K}
        outputs[f"{prec}_K{K}"] = (sums, llh)
        eng.close()
    wl.close()
    return out, {"config": "c1", "points": pts, "outputs": outputs}


def c3_sweep(local, steps=20, warmup=3):
    """Batched reweighting of the 100k-event C1 workload: LLH evaluations/s at
    K = 16, 64, 256 points per launch (FP32 dials, FP64 sums and LLH, the
    launch chain captured in a CUDA graph, shape autotuned per K).  Device
    parameters, CUDA events on the engine's stream."""
    import torch

    from gundam_gb300 import Engine, Workload

    wl = Workload("c1", seed=2)
    out = {"workload": f"c1: {wl.n_events} events, {wl.n_dials} dials, {wl.n_bins} bins, {wl.n_params} params",
           "note": "the C1 payload (~10 MB) is L2-resident"}
    check = {"config": "c1", "points": {}, "outputs": {}}
    for K in (16, 64, 256):
        eng = Engine.from_workload(wl, precision="fp32", k_max=K, llh_type=llh_type_for("c1"), device=local)
        eng.autotune(K)
        eng.use_graph(True)
        pts = torch.from_numpy(wl.draw_points(K, 7)).cuda()
        s = torch.empty((K, wl.n_bins), dtype=torch.float64, device="cuda")
        s2 = torch.empty_like(s)
        ll = torch.empty(K, dtype=torch.float64, device="cuda")
        stream = torch.cuda.Stream()
        sp = stream.cuda_stream
        for _ in range(warmup):
            eng.eval_device(pts.data_ptr(), K, s.data_ptr(), s2.data_ptr(), ll.data_ptr(), 0, sp)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            eng.eval_device(pts.data_ptr(), K, s.data_ptr(), s2.data_ptr(), ll.data_ptr(), 0, sp)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / steps
        eng.sync()
        out[f"K{K}"] = {"evals_per_s": K * 1e3 / ms, "ms_per_launch": ms, "shape": list(eng.shape())}
        check["points"][f"K{K}"] = pts.cpu().numpy()
        check["outputs"][f"K{K}"] = (s.cpu().numpy(), ll.cpu().numpy())
        eng.close()
    wl.close()
    out["error_against"] = "the CPU propagation (FP64) of the same K points (FP32 dials, FP64 sums and LLH)"
    return out, check


def mcmc_comparison(args):
    """ESS/s of the surrogate delayed-acceptance sampler against the plain
    engine sampler on this GPU (64 chains, the same start states, the same
    number of steps; the plain sampler's random walk uses the adaptive
    pilot's proposal), with a short training of the surrogate.  Stage 1 is
    Hamiltonian Monte Carlo on the surrogate (its device gradient) by
    default, random-walk sub-chains with --mcmc-stage1 rwm; the exact engine
    corrects every stage-1 proposal.  See gundam_gb300/da_mcmc.py."""
    from gundam_gb300 import da_mcmc

    r = da_mcmc.run(events=args.events, train=args.mcmc_train, epochs=args.mcmc_epochs, steps=args.mcmc_steps,
                    n_sub=args.mcmc_nsub, seed=args.seed, config=args.config, precision=args.precision,
                    linear=True, base_only_steps=args.mcmc_base_only_steps, lr=2e-3, thin=2,
                    stage1=args.mcmc_stage1)
    p, d = r["plain"], r["delayed"]
    return {
        "metric": "ESS/s, surrogate delayed acceptance vs plain engine MCMC (same GPU)",
        "unit": "effective samples/s", "higher_is_better": True,
        "plain_ess_per_s": {"min": p["ess_per_s_min"], "median": p["ess_per_s_median"]},
        "delayed_ess_per_s": {"min": d["ess_per_s_min"], "median": d["ess_per_s_median"]},
        "gain": {"min": r["ess_per_s_gain_min"], "median": r["ess_per_s_gain_median"]},
        "stage2_accept": d["stage2_accept"], "plain_accept": p["accept"], "fell_back_at_step": d["fell_back_at_step"],
        "surrogate_llh_error_sd": r["surrogate_llh_error_sd"], "posterior": r["posterior"],
        "chains": r["chains"], "steps_each": r["plain_steps"], "stage1": r["stage1"],
        "seconds": {"plain": p["seconds"], "delayed": d["seconds"], "pilot": r["pilot"]["seconds"],
                    "training_data": r["training"]["data_seconds"], "training": r["training"]["train_seconds"],
                    "total": r["total_seconds"]},
        "training": {"points": r["training"]["points"], "epochs": r["training"]["epochs"],
                     "loss_first_last": r["training"]["loss_first_last"]},
        "ess": "multi-chain (Vehtari et al. 2021) with Geyer's initial monotone sequence; chains of this length "
               "underestimate the plain sampler's autocorrelation time, so the gain here is a lower estimate",
        "network_gain": {"base_only_ess_per_s_median": r.get("delayed_base_only", {}).get("ess_per_s_median"),
                         "base_only_steps": args.mcmc_base_only_steps,
                         "delayed_over_base_only_median": r.get("network_gain_ess_per_s_median")},
        "config_departures": {
            "steps_each": f"{r['plain_steps']} (stated: 100000; the full-length run is recorded in "
                          "profiles/c4_da_mcmc_full.md)" if r["plain_steps"] != 100000 else None,
            "training_points": None if r["training"]["points"] == 1 << 20 else r["training"]["points"],
            "epochs": None if r["training"]["epochs"] == 20 else r["training"]["epochs"],
            "proposal": "the adaptive pilot's covariance and scale (GUNDAM's SimpleMcmc adaptive proposal), not "
                        "2.38^2/200 x the prior covariance: at 5M events the posterior is ~5x narrower than "
                        "the prior and that proposal accepts ~0.6 %",
            "training_region": "the pilot's posterior mean and covariance inflated x1.5, not the prior inflated "
                               "x1.5: a surrogate trained on prior draws errs by ~800 in -2 log L at posterior "
                               "states",
            "stage1": "Hamiltonian Monte Carlo on the surrogate (10 leapfrog steps) instead of one random-walk "
                      "step per stage-2 correction" if r["stage1"]["kind"] == "hmc" else None,
        },
    }


def run_gw(args, world, rank, local, dist):
    import numpy as np
    import torch

    import ctypes as C

    from gundam_gb300 import Engine, Workload
    from gundam_gb300 import _native as N
    from gundam_gb300.roofline import algorithmic_bytes, algorithmic_flops

    torch.cuda.set_device(local)
    wl = Workload(args.config, n_events=args.events, seed=args.seed)
    K = args.points
    eng = Engine.from_workload(wl, precision=args.precision, k_max=max(K, 1), llh_type=llh_type_for(args.config),
                               device=local)
    if K > 1:
        eng.autotune(K)
    pts = wl.draw_points(K, 1234 + rank)
    d = {"p": torch.from_numpy(pts).cuda(), "s": torch.empty((K, wl.n_bins), dtype=torch.float64, device="cuda")}
    d["s2"] = torch.empty_like(d["s"])
    d["l"] = torch.empty(K, dtype=torch.float64, device="cuda")

    clocks = ClockSampler(local)
    clocks.start()
    ms, kernel_ms, launches = time_device(eng, torch, d, K, args.steps, args.warmup, dist)
    clk = clocks.stop()
    ms = max_over_ranks(ms, dist)
    value = whole_job_rate(K, world, ms / 1e3)

    # e2e through the public API with host buffers (params H2D, bins + LLH D2H each step)
    for _ in range(2):
        eng.eval(pts)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.eval(pts)
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, dist)
    e2e = {"value": whole_job_rate(K, world, e2e_s), "unit": "evals/s", "h2d_bytes_per_step": K * wl.n_params * 8,
           "d2h_bytes_per_step": K * wl.n_bins * 16 + K * 16, "ms_per_step": e2e_s * 1e3}

    peak, peak_kind = peaks()
    alg = algorithmic_bytes(wl, args.precision, K)
    achieved = alg / (kernel_ms / 1e3) / 1e9
    # the batched kernels serve K points per byte read: their binding
    # resource is FP32 throughput, measured here with an FMA probe
    fp32_peak = C.c_double(0.0)
    N.libgw().gw_measure_fp32_peak(local, C.byref(fp32_peak))
    flops = algorithmic_flops(wl, K)
    compute = {"bound": "fp32", "unit": "TFLOP/s", "achieved": flops / (kernel_ms / 1e3) / 1e12,
               "peak": fp32_peak.value, "peak_source": "measured on this GPU (FMA probe, gw_measure_fp32_peak)",
               "frac": (flops / (kernel_ms / 1e3) / 1e12) / fp32_peak.value if fp32_peak.value > 0 else None,
               "algorithmic_flops_per_launch": flops}
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        tr = json.loads(tfile.read_text())
        key = f"{args.config}/{args.precision}/K{K}"
        if key in tr:
            traffic = tr[key]
    layout = eng.layout()
    shape = eng.shape()
    sidx = eng.shape_index()
    sfull = Engine.compiled_shapes()[sidx] if sidx >= 0 else None
    plain_name = PLAIN_NAMES[eng.plain_kernel()]
    variants = {}
    if not args.no_variants:
        # K = 1 (the plain kernel) on this engine, whose splines are stored in
        # the batched kernel's form (the grid form at K >= 16), and on a K = 1
        # engine (knot values)
        eng.autotune(1)
        ms1, kms1, _ = time_device(eng, torch, d, 1, args.steps, args.warmup, dist)
        variants[f"{args.precision}_K1_batched_layout"] = {"kernel": PLAIN_NAMES[eng.plain_kernel()],
            "evals_per_s": 1e3 / ms1, "ms_per_eval": ms1, "kernel_ms": kms1,
            "kernel_gbs": algorithmic_bytes(wl, args.precision, 1) / (kms1 / 1e3) / 1e9,
            "payload_bytes": layout["payload_bytes"]}
        e1 = Engine.from_workload(wl, precision=args.precision, k_max=1, llh_type=llh_type_for(args.config),
                                  device=local)
        e1.autotune(1)
        ms1, kms1, _ = time_device(e1, torch, d, 1, args.steps, args.warmup, dist)
        variants[f"{args.precision}_K1"] = {"kernel": PLAIN_NAMES[e1.plain_kernel()],
            "evals_per_s": 1e3 / ms1, "ms_per_eval": ms1, "kernel_ms": kms1,
            "kernel_gbs": algorithmic_bytes(wl, args.precision, 1) / (kms1 / 1e3) / 1e9,
            "kernel_frac_of_hbm_peak": algorithmic_bytes(wl, args.precision, 1) / (kms1 / 1e3) / 1e9 / peak,
            "payload_bytes": e1.layout()["payload_bytes"], "spline_layout": "knots"}
        e1.close()
        # small K: an engine sized for it (k_max = 4, its default spline form),
        # the warp-specialised small-K kernels, autotuned; e2e through gw_eval
        # with host buffers
        es = Engine.from_workload(wl, precision=args.precision, k_max=4, llh_type=llh_type_for(args.config),
                                  device=local)
        for Ks in (2, 4):
            es.autotune(Ks)
            msk, kmsk, _ = time_device(es, torch, d, Ks, args.steps, args.warmup, dist)
            pk = pts[:Ks]
            for _ in range(2):
                es.eval(pk)
            t0 = time.perf_counter()
            for _ in range(args.steps):
                es.eval(pk)
            e2e_k = (time.perf_counter() - t0) / args.steps
            algk = algorithmic_bytes(wl, args.precision, Ks)
            sk = es.shape_index()
            variants[f"{args.precision}_K{Ks}"] = {
                "shape": list(Engine.compiled_shapes()[sk]), "evals_per_s": Ks * 1e3 / msk, "ms_per_step": msk,
                "kernel_ms": kmsk, "kernel_gbs": algk / (kmsk / 1e3) / 1e9,
                "kernel_frac_of_hbm_peak": algk / (kmsk / 1e3) / 1e9 / peak,
                "e2e_evals_per_s": Ks / e2e_k, "e2e_ms_per_step": e2e_k * 1e3,
                "payload_bytes": es.layout()["payload_bytes"]}
        es.close()
        if K > 16:
            # C3 at the C2 size: K = 16 and K = 256 on engines sized for them
            # (each with its default spline form)
            e16 = Engine.from_workload(wl, precision=args.precision, k_max=16, llh_type=llh_type_for(args.config),
                                       device=local)
            e16.autotune(16)
            ms16, kms16, _ = time_device(e16, torch, d, 16, args.steps, args.warmup, dist)
            variants[f"{args.precision}_K16"] = {"evals_per_s": 16e3 / ms16, "ms_per_step": ms16, "kernel_ms": kms16,
                                                  "shape": list(e16.shape())}
            e16.close()
        if args.precision == "fp32":
            # the reference's precision (FP64) and the double-float mode (two
            # FP32 words per value on the FP32 pipe, sums and LLH in FP64, held
            # to the FP64 parity bar): K = 1 on a K = 1 engine, K points on an
            # engine sized for them, each with its default spline form
            for prec in ("fp64", "df64"):
                eng.close()
                eng = Engine.from_workload(wl, precision=prec, k_max=1, llh_type=llh_type_for(args.config),
                                           device=local)
                eng.autotune(1)
                ms1, kms1, _ = time_device(eng, torch, d, 1, args.steps, args.warmup, dist)
                alg1 = algorithmic_bytes(wl, prec, 1)
                variants[f"{prec}_K1"] = {"kernel": PLAIN_NAMES[eng.plain_kernel()],
                    "evals_per_s": 1e3 / ms1, "ms_per_eval": ms1, "kernel_ms": kms1,
                    "kernel_gbs": alg1 / (kms1 / 1e3) / 1e9, "kernel_frac_of_hbm_peak": alg1 / (kms1 / 1e3) / 1e9 / peak,
                    "payload_bytes": eng.layout()["payload_bytes"]}
                if K > 1:
                    eng.close()
                    eng = Engine.from_workload(wl, precision=prec, k_max=K, llh_type=llh_type_for(args.config),
                                               device=local)
                    eng.autotune(K)
                    msk, kmsk, _ = time_device(eng, torch, d, K, min(args.steps, 20), args.warmup, dist)
                    variants[f"{prec}_K{K}"] = {"evals_per_s": K * 1e3 / msk, "ms_per_step": msk, "kernel_ms": kmsk,
                                                "shape": list(Engine.compiled_shapes()[eng.shape_index()]),
                                                "payload_bytes": eng.layout()["payload_bytes"]}
            if K < 256:
                eng.close()
                K2 = 256
                eng = Engine.from_workload(wl, precision=args.precision, k_max=K2,
                                           llh_type=llh_type_for(args.config), device=local)
                eng.autotune(K2)
                d2 = {"p": torch.from_numpy(wl.draw_points(K2, 4321 + rank)).cuda(),
                      "s": torch.empty((K2, wl.n_bins), dtype=torch.float64, device="cuda")}
                d2["s2"] = torch.empty_like(d2["s"])
                d2["l"] = torch.empty(K2, dtype=torch.float64, device="cuda")
                ms2, kms2, _ = time_device(eng, torch, d2, K2, max(3, min(args.steps, 20) // 4), args.warmup, dist)
                variants[f"{args.precision}_K{K2}"] = {"evals_per_s": K2 * 1e3 / ms2, "ms_per_step": ms2,
                                                        "kernel_ms": kms2, "shape": list(eng.shape())}
        eng.sync()
    eng.close()

    cpu = None
    if rank == 0:
        v, cores, n, dt = cpu_baseline(wl, args.config, args.cpu_seconds)
        cpu = {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
               "sample": f"{n} full evaluations (K=1) of all {wl.n_events} events, {dt:.1f} s"}
        # the same on one core (the reference's event loop split over threads
        # scales with cores; the single-core rate shows the per-core cost)
        v1, _, n1, dt1 = cpu_baseline(wl, args.config, max(1.0, args.cpu_seconds / 4), threads=1)
        cpu["one_core"] = {"value": v1, "sample": f"{n1} full evaluations on 1 thread, {dt1:.1f} s"}
    if cpu:
        for key, var in variants.items():
            if "e2e_evals_per_s" in var:
                var["e2e_over_cpu_baseline"] = var["e2e_evals_per_s"] / cpu["value"]
    c3 = c1 = c5 = None
    c1_check = c3_check = c5_check = None
    if rank == 0 and not args.no_variants:
        c3, c3_check = c3_sweep(local)
        c1, c1_check = c1_points(local)
    if rank == 0 and not args.no_c5 and args.config == "c2":
        from gundam_gb300 import stress

        # progress to stderr: stdout carries the one JSON line
        c5 = stress.run(check_points=2, log=lambda m: print(m, file=sys.stderr, flush=True))
        c5_check = c5.pop("check", None)
    if rank == 0 and (c1_check or c3_check or c5_check):
        chk = cpu_baseline_checks(c1_check, c3_check, c5_check)
        if c1 is not None and "c1" in chk:
            for key, v in chk["c1"].items():
                if isinstance(v, dict):
                    c1[key].update(v)
                else:
                    c1[key] = v
        if c3 is not None and "c3" in chk:
            for key, v in chk["c3"].items():
                c3[key].update(v)
        if c5 is not None and "c5" in chk:
            c5["parity_against_cpu_propagation"] = chk["c5"]
    mc = None
    if rank == 0 and not args.no_mcmc and args.config == "c2":
        mc = mcmc_comparison(args)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 dials / f64 sums" if args.precision == "fp32" else "f64",
            "data": "synthetic (seeded generator, C2 shapes)",
            "config": {"workload": f"{args.config}: {wl.n_events} events, {wl.n_dials} dials, "
                                   f"{wl.n_bins} bins, {wl.n_params} params",
                       "points_per_step": K, "precision": args.precision, "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas x{world}", "tiles": layout["n_tiles"],
                       "payload_bytes": layout["payload_bytes"],
                       "kernel_shape": {"family": shape[0], "points_per_pass": shape[1], "threads": shape[2],
                                        "stages": shape[3], "index": sidx,
                                        "points_per_thread": sfull[2] if sfull else None,
                                        "min_blocks_per_sm": sfull[5] if sfull else None}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "binding": ("compute" if compute["frac"] and compute["frac"] > achieved / peak else "hbm"),
                         "kernel": (plain_name if K == 1 else ("k_multi" if shape[0] == 1 else "k_batched")),
                         "kernel_ms": kernel_ms,
                         "algorithmic_bytes_per_launch": alg, "compute": compute},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk,
            "variants": variants,
            "event_dials_per_s": value * wl.n_dials,
            "c3_batched_vs_k": c3,
            "c1_thousand_points": c1,
            "c5_stress": c5,
            "mcmc": mc,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()


def main():
    args = parse()
    world, rank, local, dist = dist_setup(args)
    try:
        if args.impl == "reference":
            run_reference(args, world, rank, dist)
        else:
            run_gw(args, world, rank, local, dist)
    finally:
        if dist is not None and dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
