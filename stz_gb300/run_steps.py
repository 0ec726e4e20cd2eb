"""Run a few quasi-static steps of the simple-shear configuration on the GPU.

    python -m stz_gb300.run_steps --size 2048 --precision mixed --warmup 1 --steps 2

Prints ms/step and multigrid statistics.  This is the command the profiles
under profiles/ were captured with (ncu wraps it).
"""
import argparse
import time

from . import _lib
from .params import simple_shear
from .shear_sim import ShearSim, random_chi


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--std", type=float, default=40.0)
    ap.add_argument("--corr", type=float, default=16.0)
    ap.add_argument("--no-extrapolate", action="store_true")
    ap.add_argument("--direct", action="store_true", help="explicit steps (dt = dx^2/2) instead of quasi-static")
    ap.add_argument("--time-kernels", action="store_true",
                    help="after the steps, time the kernel groups of stzg_time_kernel (advection, projection "
                         "source, FP32 V-cycle, outer residual, stress correction) with CUDA events")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch every kernel from the host (a profiler then lists the solve's kernels too; "
                         "the solve follows the host-side refinement policy)")
    a = ap.parse_args(argv)
    N = a.size
    P = simple_shear(N)
    chi = random_chi(N, N, a.corr, 600.0, a.std, P.TZ, 2)
    prec = _lib.MIXED if a.precision == "mixed" else _lib.FP64
    sim = ShearSim(P, chi, precision=prec, tol_mode=_lib.TOL_RELATIVE, tol=a.tol,
                   extrapolate=not a.no_extrapolate, use_graphs=not a.no_graphs)
    if a.direct:
        ddt = 0.5 * (2.0 / N) ** 2
        sim.step_forward(ddt, a.warmup)
        t0 = time.time()
        sim.step_forward(ddt, a.steps)
        t = time.time() - t0
        print(f"N={N} explicit: {1e3 * t / max(a.steps, 1):.2f} ms/step, {sim.stats.kernel_launches} kernels")
        sim.close()
        return
    sim.steps(1e-2, a.warmup)
    t0 = time.time()
    sim.steps(1e-2, a.steps)
    t = time.time() - t0
    st = sim.stats
    print(f"N={N} {a.precision}: {1e3 * t / max(a.steps, 1):.2f} ms/step, {st.vcycles / max(a.steps, 1):.1f} "
          f"V-cycles/step (+{st.extra_vcycles / max(a.steps, 1):.1f} after convergence), {st.refinements / max(a.steps, 1):.1f} passes/step, {st.kernel_launches} kernels")
    if a.time_kernels:
        ids = [(0, "advection"), (8, "projection source")]
        if prec == _lib.MIXED:
            ids += [(4, "FP32 V-cycle"), (5, "outer residual (float-float) + norms")]
        else:
            ids += [(3, "FP64 V-cycle")]
        ids += [(9, "stress correction + wall rows (changes the stresses)")]
        for k, name in ids:
            print(f"  {name}: {sim.time_kernel(1e-2, k, 10):.4f} ms")
    sim.close()


if __name__ == "__main__":
    main()
