"""A small, self-contained case for profiling one kernel under ncu.

    python -m gundam_gb300.profile_case {plain|batched} {fp32|fp64} [n_events]

Builds the C2-shaped workload with n_events events (default 1,000,000: a
payload above the 129 MB L2 but a few GB of device memory at most) and
evaluates it four times: K = 1 (k_plain) or K = 64 with the batched shape the
benchmark selects on this workload (k_batched, 64 points per pass, 256
threads, one payload stage).  Profile with e.g.
    ncu --set full --clock-control none -k regex:k_plain -s 2 -c 1 ...
"""
import sys

from .engine import Engine
from .workload import Workload


def main(argv):
    mode, precision = argv[0], argv[1]
    n = int(argv[2]) if len(argv) > 2 else 1000000
    wl = Workload("c2", n_events=n, seed=2)
    K = 64 if mode == "batched" else 1
    eng = Engine.from_workload(wl, precision=precision, k_max=64)
    if mode == "batched":
        eng.set_shape(0, 64, 256, 1)
    pts = wl.draw_points(K, 5)
    for _ in range(4):
        eng.eval(pts)
    print("ok", eng.layout()["payload_bytes"], eng.shape())


if __name__ == "__main__":
    main(sys.argv[1:])
