"""Run the batched configuration: many independent simulations of uneven
grid sizes advanced together in one CUDA graph.

    python -m stz_gb300.run_batch --count 256 --steps 100 --precision mixed --autotune
"""
import argparse
import json
import time

from . import _lib
from .batch import Batch, batched_config


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--tune-steps", type=int, default=4)
    a = ap.parse_args(argv)
    params, chis = batched_config(a.count)
    prec = _lib.MIXED if a.precision == "mixed" else _lib.FP64
    t0 = time.time()
    b = Batch(params, chis, precision=prec, tol=a.tol)
    setup = time.time() - t0
    tuned = None
    if a.autotune:
        t0 = time.time()
        tuned = {f"{m}x{n}": v for (m, n), v in b.autotune(1e-2, a.tune_steps).items()}
        tune_s = time.time() - t0
    t0 = time.time()
    st = b.run(1e-2, a.steps)
    wall = time.time() - t0
    out = {"workload": f"{a.count} simple-shear simulations, grids 64..512 squared, {a.steps} steps, one CUDA graph",
           "precision": a.precision, "cell_steps_per_s": st.cell_steps / st.seconds, "graph_seconds": st.seconds,
           "wall_seconds": wall, "vcycles": st.vcycles, "passes": st.passes, "failed": st.failed,
           "graph_kernels": st.graph_kernels, "kernel_launches": st.kernel_launches, "setup_s": setup,
           "cells": sum(p.m * p.n for p in params)}
    if tuned:
        out["tuning"] = tuned
        out["tune_s"] = tune_s
    print(json.dumps(out))
    b.close()


if __name__ == "__main__":
    main()
