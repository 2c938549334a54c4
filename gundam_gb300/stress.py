"""The large-scale stress configuration (C5) on one GPU.

    python -m gundam_gb300.stress [--events N] [--precisions fp32,fp64]

40M events in 12 samples (10,000 bins), 400 parameters, ~10 spline/graph
dials per event plus one kriged dial per event reading a 4096-entry table
that the engine recomputes on the device from six parameters before every
evaluation.  For each precision: the build (generation, cache building,
packing and upload), the resident device memory and the high-water mark of
the device's used memory, and the time per pass of the plain kernel (K = 1)
and of the batched kernels (K = 64, autotuned), with the achieved HBM
bandwidth of the algorithmic bytes against the measured peak.

Host memory: the workload (~60 GB at 40M events) is released after the
engine has copied it and before the cache is packed, so the peak stays near
the workload plus the engine's copy (~125 GB); the run stops before starting
if the host has less available memory than that estimate.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import time
from pathlib import Path

from .engine import Engine
from .roofline import algorithmic_bytes
from .workload import Workload

ROOT = Path(__file__).resolve().parents[1]


def host_available_gb() -> float:
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return float(line.split()[1]) / 1e6
    except OSError:
        pass
    return float("nan")


def device_used_gb(torch) -> float:
    free, total = torch.cuda.mem_get_info()
    return (total - free) / 1e9


def time_eval(eng, torch, K, pts_dev, outs, steps=5, warmup=2):
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    s, s2, ll = outs
    for _ in range(warmup):
        eng.eval_device(pts_dev.data_ptr(), K, s.data_ptr(), s2.data_ptr(), ll.data_ptr(), 0, sp)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        eng.eval_device(pts_dev.data_ptr(), K, s.data_ptr(), s2.data_ptr(), ll.data_ptr(), 0, sp)
    b.record(stream)
    torch.cuda.synchronize()
    eng.sync()
    return a.elapsed_time(b) / steps


def run(events=40_000_000, precisions=("fp32", "fp64"), seed=2, log=print, check_points=0):
    """check_points > 0: the engine's bin sums and likelihood at the first
    check_points parameter points (the K = 1 kernel at the first one, the
    K = 64 batched shape at all of them) are returned under "check", with the
    points and the workload's size and seed, for a comparison with the CPU
    propagation of the same workload."""
    import torch

    peak_bw = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"] \
        if (ROOT / "MEASURED_PEAKS.json").exists() else 6800.0
    need = 3.2 * events / 2e6 * 2.1  # GB: workload + the engine's copy
    avail = host_available_gb()
    if avail == avail and avail < need:
        return {"skipped": f"host has {avail:.0f} GB available, the build needs ~{need:.0f} GB"}
    out = {"events": events, "host_available_gb": avail, "peak_hbm_gbs": peak_bw}
    check = {"events": events, "seed": seed, "outputs": {}} if check_points > 0 else None
    torch.cuda.init()
    base_used = device_used_gb(torch)
    for prec in precisions:
        r = {}
        t0 = time.perf_counter()
        wl = Workload("c5", n_events=events, seed=seed)
        r["generate_s"] = time.perf_counter() - t0
        meta = {"events": wl.n_events, "dials": wl.n_dials, "bins": wl.n_bins, "params": wl.n_params,
                "tables": wl.n_tables}
        bytes1 = algorithmic_bytes(wl, prec, 1)
        bytes64 = algorithmic_bytes(wl, prec, 64)
        pts = wl.draw_points(64, 11)
        if check is not None:
            check["points"] = pts[:check_points]
        t0 = time.perf_counter()
        eng = Engine.from_workload(wl, precision=prec, k_max=64, initialize=False)
        r["cache_build_s"] = time.perf_counter() - t0
        wl.close()
        del wl
        gc.collect()
        t0 = time.perf_counter()
        eng.initialize()
        r["pack_upload_s"] = time.perf_counter() - t0
        hw = device_used_gb(torch) - base_used
        r["resident_bytes"] = eng.resident_memory()
        p_dev = torch.from_numpy(pts).cuda()
        outs = (torch.empty((64, meta["bins"]), dtype=torch.float64, device="cuda"),
                torch.empty((64, meta["bins"]), dtype=torch.float64, device="cuda"),
                torch.empty(64, dtype=torch.float64, device="cuda"))
        eng.autotune(1)
        ms1 = time_eval(eng, torch, 1, p_dev, outs)
        if check is not None:
            s1, _, l1, _ = eng.eval(pts[:1])
            check["outputs"][f"{prec}_K1"] = (s1.copy(), l1.copy())
        hw = max(hw, device_used_gb(torch) - base_used)
        r["plain_K1"] = {"ms_per_pass": ms1, "evals_per_s": 1e3 / ms1,
                         "hbm_gbs": bytes1 / (ms1 / 1e3) / 1e9, "frac": bytes1 / (ms1 / 1e3) / 1e9 / peak_bw,
                         "algorithmic_bytes": bytes1,
                         "kernel": ["k_plain", "k_plain_ws", "k_plain_ws (8 evaluator warps)"][eng.plain_kernel()]}
        eng.autotune(64)
        ms64 = time_eval(eng, torch, 64, p_dev, outs)
        if check is not None:
            sk, _, lk, _ = eng.eval(pts[:check_points])
            check["outputs"][f"{prec}_batched"] = (sk.copy(), lk.copy())
        hw = max(hw, device_used_gb(torch) - base_used)
        r["batched_K64"] = {"ms_per_pass": ms64, "evals_per_s": 64e3 / ms64,
                            "hbm_gbs": bytes64 / (ms64 / 1e3) / 1e9, "shape": list(eng.shape()),
                            "shape_entry": list(Engine.compiled_shapes()[eng.shape_index()]),
                            "algorithmic_bytes": bytes64}
        r["device_memory_high_water_gb"] = hw
        r.update(meta)
        out[prec] = r
        log(f"{prec}: {json.dumps(r)}")
        eng.close()
        del eng, p_dev, outs
        gc.collect()
        torch.cuda.empty_cache()
    if check is not None:
        out["check"] = check
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--events", type=int, default=40_000_000)
    ap.add_argument("--precisions", default="fp32,fp64")
    a = ap.parse_args()
    print(json.dumps(run(a.events, tuple(a.precisions.split(",")), log=lambda m: print(m, flush=True))))


if __name__ == "__main__":
    main()
