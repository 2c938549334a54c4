"""A small, self-contained case for profiling one kernel under ncu.

    python -m gundam_gb300.profile_case {plain|batched} {fp32|fp64|df64} [n_events] [shape_index] [K]
    python -m gundam_gb300.profile_case train [steps]
    python -m gundam_gb300.profile_case substeps [n_sub]

plain / batched: builds the C2-shaped workload with n_events events (default
1,000,000: a payload above the 129 MB L2 but a few GB of device memory at
most) and evaluates it four times: K = 1 (the K = 1 kernel the autotuner
picks, on a K = 1 engine: Catmull-Rom splines stored as knot values in FP32;
the autotuner's launches come before the four) or K points
(default 64) with batched shape `shape_index` (an entry of
Engine.compiled_shapes(); -1 or none: the autotuner picks one first, and the
chosen index is printed).

train: the C2 surrogate network (200 -> 512 -> 512 -> 512 -> 3000, BF16)
trained for `steps` (default 8) Adam steps of batch 2048 on a device-resident
set of 8192 random points (the tcgen05 GEMMs k_gemm, the loss, Adam).

substeps: 64 surrogate sub-chains of n_sub (default 4) steps with an additive
head fitted to a synthetic response (k_propose, the GEMMs, k_head_llh,
k_penalty, k_accept).

Profile with e.g.
    ncu --set full --clock-control none -k regex:k_plain -s 2 -c 1 ...
"""
import sys

import numpy as np

from . import _native as N
from .engine import Engine
from .workload import Workload


def _surrogate(P=200, B=3000, seed=0):
    from .surrogate import Surrogate

    rng = np.random.default_rng(seed)
    th = rng.standard_normal((4096, P)) * 0.2
    logs = 5.0 + th @ rng.normal(0, 0.05, (P, B)) + 0.01 * np.sin(th[:, :1] * 3.0)
    sur = Surrogate(P, B, batch_max=4096, seed=seed + 1)
    sur.fit_additive(th, logs, log_ratio=np.zeros_like(logs) + 0.1 * th[:, :1], nodes=8)
    sur.attach(np.round(np.exp(logs[0])), None, N.GW_LLH_BARLOW_BEESTON_OA2021)
    return sur, th, logs


def main(argv):
    mode = argv[0]
    if mode == "train":
        steps = int(argv[1]) if len(argv) > 1 else 8
        sur, th, logs = _surrogate()
        sur.reserve(8192)
        sur.append(th, np.exp(logs))
        sur.append(th, np.exp(logs))
        h = sur.train(epochs=max(1, steps // 4), batch=2048)
        print("ok", h)
        return
    if mode == "substeps":
        n_sub = int(argv[1]) if len(argv) > 1 else 4
        sur, th, _ = _surrogate()
        P = th.shape[1]
        sur.set_chain(np.linalg.cholesky(np.eye(P) * 1e-3), np.zeros(P), np.eye(P))
        _, f0, _ = sur.substeps(th[:64], None, 0, 1)
        for r in range(3):
            _, _, nacc = sur.substeps(th[:64], f0, n_sub, 10 + r)
        print("ok", float(nacc.mean()))
        return
    precision = argv[1]
    n = int(argv[2]) if len(argv) > 2 else 1000000
    wl = Workload("c2", n_events=n, seed=2)
    K = (int(argv[4]) if len(argv) > 4 else 64) if mode == "batched" else 1
    eng = Engine.from_workload(wl, precision=precision, k_max=max(K, 64) if mode == "batched" else 1)
    if mode == "batched":
        if len(argv) > 3 and int(argv[3]) >= 0:
            eng.set_shape_index(int(argv[3]))
        else:
            eng.autotune(K)
    else:
        eng.autotune(1)  # the K = 1 kernel kind the engine would pick
    pts = wl.draw_points(K, 5)
    for _ in range(4):
        eng.eval(pts)
    print("ok", eng.layout()["payload_bytes"], eng.shape(), "shape index", eng.shape_index(),
          "K = 1 kernel", eng.plain_kernel())


if __name__ == "__main__":
    main(sys.argv[1:])
