"""Timing harness of the general multigrid: the pfd_time.cc loop
(esim/tgmg/pfd_time.cc:14-81) on the GPU.

poisson_fd on a 2049 x 2049 grid over [-8,8]^2; each trial moves a Gaussian
source (radius 1) along a circle of radius 6 through one turn and solves with
solve_v_cycle(tgmg_predict&).  Prints one JSON line: wall and device time per
solve (the wall time includes the copies of b in and z out that the mirror of
the reference's in-place arrays makes), V-cycles per solve, device time per
V-cycle and its algorithmic HBM bandwidth.

    python -m stz_gb300.run_pfd [--size 2049] [--trials 500] [--precision fp64|mixed]

With --precision mixed each "V-cycle" is a refinement pass (an FP32 V-cycle
on the FP64 residual, the correction added in FP64), and the bandwidth
figure is left out (the pass moves different bytes).
"""
import argparse
import json
import math
import time

import numpy as np

from . import tgmg

# Algorithmic bytes of one FP64 V-cycle per fine point, cyc_down = cyc_up = 1:
# per level a pre-sweep and a post-sweep (read z, b and the 4-byte stencil
# index, write z: 28 B each), the residual (read z, b, index, write r: 28 B),
# the restriction (read r: 8 B) and the prolongation (read and write z: 16 B),
# 108 B, times 4/3 for the coarser levels.
VCYCLE_BYTES_PER_POINT = 108 * 4 / 3


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=2049)
    ap.add_argument("--trials", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    args = ap.parse_args(argv)
    m = n = args.size
    q = tgmg.PoissonFD(m, n, -8.0, 8.0, -8.0, 8.0)
    g = tgmg.Tgmg(q)
    mixed = args.precision == "mixed"
    g.set_precision(mixed)
    tp = tgmg.Predict()
    h = 2.0 * math.pi / args.trials
    for k in range(args.warmup):
        q.gaussian_source_term(6 * math.cos(h * k), 6 * math.sin(h * k), 1, 1)
        assert g.solve_v_cycle(tp)
    tp.solves = tp.vcount = 0
    wall = dev = 0.0
    kernels = 0
    for k in range(args.trials):
        q.gaussian_source_term(6 * math.cos(h * k), 6 * math.sin(h * k), 1, 1)
        t0 = time.perf_counter()
        ok = g.solve_v_cycle(tp)
        wall += time.perf_counter() - t0
        assert ok
        ms, kn = g.last_timing()
        dev += ms * 1e-3
        kernels += kn
    vc = tp.vcount + tp.extra_iters * tp.solves
    per_v = dev / max(vc, 1)
    line = {"workload": "poisson_fd %dx%d on [-8,8]^2, rotating Gaussian source, solve_v_cycle(tgmg_predict&)" % (m, n),
            "trials": args.trials, "wall_ms_per_solve": 1e3 * wall / args.trials,
            "device_ms_per_solve": 1e3 * dev / args.trials,
            "vcycles_per_solve": tp.vcount / tp.solves, "extra_vcycles_per_solve": tp.extra_iters,
            "device_ms_per_vcycle": 1e3 * per_v,
            "vcycle_algorithmic_GBs": None if mixed else VCYCLE_BYTES_PER_POINT * m * n / per_v / 1e9,
            "kernels_per_solve": kernels / args.trials, "levels": g.levels(),
            "final_l2_error": g.l2_error(), "acc": q.acc, "precision": args.precision}
    print(json.dumps(line))
    g.close()
    return line


if __name__ == "__main__":
    main()
