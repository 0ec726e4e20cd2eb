"""Timing harness of the step in sheared coordinates (include/stzg_ct.h): the
reference driver's configuration (shear_coord_transform.cc:20-89: Vitreloy-1
constants, linear athermal law, y periodic with lamb = 1e-3, chi_case 0)
scaled to a larger grid; warm-up steps, then timed steps of the driver's
dt = tf/600.  Prints one JSON line.

    python -m stz_gb300.run_ct [--m 2048] [--n 1024] [--steps 20] [--warmup 3] [--walls]
                               [--precision fp64|mixed] [--checked] [--direct DT] [--tracers MM NN]

--direct DT times the explicit step (shear_sim::step_forward) of dt DT
instead; --tracers MM NN adds an MM x NN tracer grid after the warm-up and
times one update_tracers after the timed steps.  --batch K times K
independent simulations of the given size (a UQ sweep: K parameter samples,
here K chi levels) stepped one after the other and then together through
stzg_ct_batch_step_qs, and prints both wall rates.
"""
import argparse
import json
import time

from .ct_sim import CtSim, transform_shear


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--m", type=int, default=2048)
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--walls", action="store_true")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64",
                    help="the projection's solve: FP64 V-cycles, or FP32 V-cycles inside FP64 refinement")
    ap.add_argument("--checked", action="store_true",
                    help="V-cycles until the residual meets the threshold instead of the reference's predicted counts")
    ap.add_argument("--direct", type=float, default=None)
    ap.add_argument("--tracers", type=int, nargs=2, default=None)
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args(argv)
    yp = not args.walls
    P = transform_shear(args.m, args.n, y_prd=yp)
    dt = (0.5 / 1e-3 if yp else 3e6 / 2e4) / 600
    if args.batch:
        return batch_main(args, P, dt, yp)
    sim = CtSim(P)
    sim.init_fields(0, 580.0, 220.0)
    sim.set_precision(args.precision == "mixed")
    sim.set_solve_policy(args.checked)
    kind = "quasi-static"
    step = sim.step_forward_quasistatic
    if args.direct:
        dt, kind, step = args.direct, "explicit", sim.step_forward
    step(dt, args.warmup)
    if args.tracers:
        sim.initialize_tracers(*args.tracers)
    t0 = time.perf_counter()
    step(dt, args.steps)
    wall = time.perf_counter() - t0
    line = {"workload": "coord_transforms simple shear %dx%d, %s, %s steps of dt %.6g" %
                        (args.m, args.n, "y periodic, lamb 1e-3" if yp else "walls", kind, dt),
            "metric": "cell-steps/s", "value": args.m * args.n * args.steps / sim.seconds,
            "ms_per_step": 1e3 * sim.seconds / args.steps, "wall_ms_per_step": 1e3 * wall / args.steps,
            "vcycles_per_step": sim.vcycles / args.steps if not args.direct else 0, "steps": args.steps,
            "warmup": args.warmup, "precision": args.precision,
            "solve": "checked" if args.checked else "predictor"}
    if args.tracers:
        t0 = time.perf_counter()
        lost = sim.update_tracers()
        line["tracers"] = {"count": len(sim.tracers()), "lost": lost,
                           "update_ms_wall": 1e3 * (time.perf_counter() - t0)}
    print(json.dumps(line))
    sim.close()
    return line


def batch_main(args, P, dt, yp):
    from .ct_sim import batch_step_qs

    def make():
        sims = []
        for k in range(args.batch):
            sim = CtSim(P)
            sim.init_fields(0, 560.0 + 40.0 * k / max(args.batch - 1, 1), 220.0)
            sim.set_precision(args.precision == "mixed")
            sim.set_solve_policy(args.checked)
            sims.append(sim)
        return sims

    sims = make()
    for s in sims:
        s.step_forward_quasistatic(dt, args.warmup)
    t0 = time.perf_counter()
    for s in sims:
        s.step_forward_quasistatic(dt, args.steps)
    seq = time.perf_counter() - t0
    for s in sims:
        s.close()
    sims = make()
    batch_step_qs(sims, dt, args.warmup, args.threads)
    _, wall = batch_step_qs(sims, dt, args.steps, args.threads)
    cells = args.m * args.n * args.steps * args.batch
    line = {"workload": "%d coord_transforms simple-shear simulations %dx%d, %s, quasi-static, %d steps of dt %.6g"
                        % (args.batch, args.m, args.n, "y periodic, lamb 1e-3" if yp else "walls", args.steps, dt),
            "metric": "cell-steps/s (wall)", "batched": cells / wall, "one_after_another": cells / seq,
            "speedup": seq / wall, "threads": args.threads or min(args.batch, 16)}
    for s in sims:
        s.close()
    print(json.dumps(line))
    return line


if __name__ == "__main__":
    main()
