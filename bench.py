#!/usr/bin/env python
"""Throughput of the quasi-static STZ time step on one or more GB300s.

Workload (the headline configuration): simple shear on a 2048x2048 grid,
periodic in x, walls at +-1e-4, mu=1, K=2.5, athermal linear STZ law,
seeded Gaussian chi (mean 600 K, std 40 K, correlation length 16 cells),
dt=1e-2, multigrid to a relative residual of 1e-10, mixed precision (FP32
V-cycles inside FP64 iterative refinement).  A step is one quasi-static time
step (advection + STZ plasticity + projection).  The ~0.6 GB FP64 state is
larger than the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  With N>1 (launched under torch.distributed.run) every
rank runs an independent replica (the step does not shard; weak scaling) and
value is the sum over ranks, timed by the slowest rank.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s"
GRID = 2048
DT = 1e-2
RTOL = 1e-10
CHI = dict(l=16.0, tem_avg=600.0, tem_std=40.0)

# Algorithmic bytes (FP64 state, FP32 multigrid vectors), per cell or node:
ADVECT_BYTES_PER_CELL = 128      # read u,v,p,q,s,tau,chi,X,Y; write p,q,s,tau,chi,X,Y (8 B each)
TOP_BYTES_PER_NODE = 26.0        # one top-level streaming kernel: 6.5 words of 4 B
VCYCLE32_BYTES_PER_NODE = 69.3   # 17.3 words of 4 B: 13 W on the top level x (1 + 1/4 + 1/16 + ...)
VCYCLE64_BYTES_PER_NODE = 138.7
SWEEP32_BYTES_PER_NODE = 24      # one Gauss-Seidel sweep: read z, b; write z (float2)
# DRAM bytes (read + write) of one launch at 2048x2048 from the committed ncu
# captures (cold caches); the advection kernel per precision
NCU_TRAFFIC_2048 = {"advect_mixed": 535.9e6, "advect_fp64": 659.8e6, "residual_ff": 153.0e6,
                    "source_mixed": 170.8e6}
SOURCE_BYTES_PER_NODE = 48       # read p,q,s,tau of the cells (8 B each, once per cell); write the source (16 B)
DIRECT_BYTES_PER_CELL = 160      # explicit step: read u,v,p,q,s,tau,chi,X,Y; write them, ddev (8 B each)
RESIDFF_BYTES_PER_NODE = 40      # read z, b as float-float (hi, lo float2 each); write r (float2)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300, help="timed steps (300: the 2048x2048 mixed-precision run)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=GRID)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-extrapolate", action="store_true")
    ap.add_argument("--extrapolate-order", type=int, default=1, choices=[1, 2],
                    help="initial guess: 1 linear, 2 quadratic extrapolation of the last solutions")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=0, help="FP64 comparison steps (0: = steps+warmup, capped)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--inner", type=int, default=0, help="FP32 V-cycles per refinement pass (0: library default)")
    ap.add_argument("--skip-extras", action="store_true", help="only the timed line (no FP64 leg, e2e, CPU)")
    ap.add_argument("--skip-batch", action="store_true", help="no batched-configuration leg")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=100)
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, ws, rank, local, backend="nccl"):
        self.ws, self.rank, self.local = ws, rank, local
        self.pg = None
        if ws > 1:
            import torch
            import torch.distributed as td
            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend=backend)
            self.td, self.torch = td, torch
            self.pg = True

    def barrier(self):
        if self.pg:
            if self.td.get_backend() == "nccl":
                self.td.barrier(device_ids=[self.local])
            else:
                self.td.barrier()

    def max(self, x):
        if not self.pg:
            return x
        dev = f"cuda:{self.local}" if self.td.get_backend() == "nccl" else "cpu"
        t = self.torch.tensor([float(x)], dtype=self.torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_params(N):
    from stz_gb300.params import simple_shear
    return simple_shear(N)


def cpu_baseline(P, chi, steps, warm=1):
    """The oracle restatement of the reference step on the host cores,
    relative residual 1e-10 like the GPU path; then one more step of the same
    run on one thread."""
    from oracle.bind import OracleSim, oracle_threads, set_oracle_threads
    t0 = time.time()
    o = OracleSim(P, chi)
    o.set_tolerance(1, RTOL)
    o.steps(DT, warm)
    o.seconds = 0.0
    o.steps(DT, steps)
    sec = o.seconds
    cores = oracle_threads()
    n = P.m * P.n
    rec = {"value": n * steps / sec, "unit": METRIC, "cores": cores, "kind": "port",
           "sample": f"{P.m}x{P.n}, {steps} timed steps after {warm} warm-up step(s), oracle restatement "
                     f"(C, OpenMP) at relative residual {RTOL:g}; set-up {time.time() - t0 - sec:.1f} s untimed",
           "ms_per_step": 1e3 * sec / steps}
    set_oracle_threads(1)
    o.seconds = 0.0
    o.steps(DT, 1)
    set_oracle_threads(cores)
    rec["one_thread"] = {"value": n / o.seconds, "unit": METRIC, "cores": 1, "ms_per_step": 1e3 * o.seconds,
                         "sample": "the next step of the same run on one thread"}
    o.close()
    return rec


PARITY_TOL = {"oracle": 1e-13, "fp64": 1e-13, "mixed": 1e-12}


def prestress(sim, tau=1.02):
    """Plastic-active start: uniform shear stress tau (units of the yield
    stress) in every cell, so every cell runs the plastic sub-stepping."""
    t = sim.get("tau")
    t[:] = tau
    sim.set("tau", t)


def parity_vs_oracle(P, chi, nsteps, extrap, plastic=False):
    """Group-normalised errors of the GPU paths against the oracle after the
    same steps from the same state.  The oracle and the GPU solve to tight
    relative residuals (the stresses are differences of the solved velocity
    over one cell, so a looser solve moves them far more than the 1e-10 gate
    in any implementation); the GPU paths at the benchmark's own tolerance
    are reported beside them."""
    from oracle.bind import OracleSim
    from stz_gb300 import _lib
    from stz_gb300.shear_sim import ShearSim
    from parity import group_errors
    o = OracleSim(P, chi)
    o.set_tolerance(1, PARITY_TOL["oracle"])
    if plastic:
        prestress(o)
    o.steps(DT, nsteps)
    ref = o.fields()
    o.close()
    out = {"steps": nsteps, "tolerances": dict(PARITY_TOL)}
    runs = (("fp64", _lib.FP64, PARITY_TOL["fp64"]), ("mixed", _lib.MIXED, PARITY_TOL["mixed"]),
            ("fp64_at_bench_tolerance", _lib.FP64, RTOL), ("mixed_at_bench_tolerance", _lib.MIXED, RTOL))
    for name, prec, tol in runs:
        g = ShearSim(P, chi, precision=prec, tol_mode=_lib.TOL_RELATIVE, tol=tol, extrapolate=extrap)
        if plastic:
            prestress(g)
        g.steps(DT, nsteps)
        out[name] = {k: float(v) for k, v in group_errors(ref, g.fields(), P.n).items()}
        g.close()
    if plastic:
        out["eps_pl_max"] = float(ref["eps_pl"].max())
    return out


def batched_leg(args):
    """The batched configuration: independent simple-shear simulations with
    grids drawn from 64..512 squared (own chi fields and STZ constants),
    advanced together in one CUDA graph after the per-size autotuner, in mixed
    precision and in FP64.  value = the batch's cell-steps over the graph's
    device time."""
    from stz_gb300 import _lib
    from stz_gb300.batch import Batch, batched_config
    params, chis = batched_config(args.batch_count)
    out = {"workload": f"{args.batch_count} simple-shear simulations, grids drawn from 64..512 squared, "
                       f"{args.batch_steps} steps of dt {DT:g}, relative residual {RTOL:g}, one CUDA graph",
           "cells": int(sum(p.m * p.n for p in params)), "unit": METRIC}
    for name, prec in (("mixed", _lib.MIXED), ("fp64", _lib.FP64)):
        b = Batch(params, chis, precision=prec, tol=RTOL)
        t0 = time.time()
        b.autotune(DT, 4)
        tune_s = time.time() - t0
        st = b.run(DT, args.batch_steps)
        out[name] = {"value": st.cell_steps / st.seconds, "graph_seconds": st.seconds,
                     "vcycles_per_instance_step": st.vcycles / (args.batch_count * args.batch_steps),
                     "failed": int(st.failed), "autotune_s": tune_s}
        b.close()
    return out


def bench_config(args, extrap, replicas):
    """The workload dict both arms print (the reference arm times the same
    workload on the host cores, in FP64)."""
    N = args.size
    mixed = args.precision == "mixed"
    return {"workload": f"quasi-static STZ simple shear {N}x{N}, "
                        f"{'FP32 V-cycles in FP64 iterative refinement' if mixed else 'FP64'} multigrid, "
                        f"relative residual {RTOL:g}",
            "grid": N, "dt": DT, "precision": args.precision, "chi": CHI, "extrapolated_guess": extrap,
            "l2": "state (~0.6 GB FP64) larger than L2; no flush", "replicas": replicas}


def run_reference(args, dist):
    """Reference arm: the reference's CPU implementation of the step on the
    host cores.  The reference's own build is compiled from its sources in
    place and is x86-only, so the C restatement of it (oracle/stz_oracle.c)
    is timed; chi comes from the oracle's own generator, so nothing of the
    product library is loaded in this process."""
    if dist.rank != 0:
        return None
    from oracle.bind import OracleSim, oracle_threads, random_chi as oracle_random_chi
    N = args.size
    P = make_params(N)
    chi = oracle_random_chi(N, N, CHI["l"], CHI["tem_avg"], CHI["tem_std"], P.TZ, 2)
    o = OracleSim(P, chi)
    o.set_tolerance(1, RTOL)
    o.steps(DT, args.warmup)
    o.seconds = 0.0
    t0 = time.time()
    o.steps(DT, args.steps)
    wall = time.time() - t0
    sec = o.seconds
    value = N * N * args.steps / sec
    extrap = 0 if args.no_extrapolate else args.extrapolate_order
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian chi, mean 600 K, std 40 K, l=16 cells)",
            "impl": "reference",
            "config": bench_config(args, extrap, int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": oracle_threads(), "kind": "port",
                             "sample": f"{args.steps} steps of {N}x{N} after {args.warmup} warm-up steps, "
                                       f"FP64 at relative residual {RTOL:g}; wall {wall:.1f} s"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


def run_ours(args, dist):
    from stz_gb300 import _lib
    from stz_gb300.shear_sim import ShearSim, random_chi
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    N = args.size
    P = make_params(N)
    chi = random_chi(N, N, CHI["l"], CHI["tem_avg"], CHI["tem_std"], P.TZ, 2 + dist.rank)
    prec = _lib.MIXED if args.precision == "mixed" else _lib.FP64
    extrap = 0 if args.no_extrapolate else args.extrapolate_order
    sim = ShearSim(P, chi, precision=prec, tol_mode=_lib.TOL_RELATIVE, tol=RTOL, device=dist.local,
                   extrapolate=extrap, inner_cycles=args.inner)
    sim.steps(DT, args.warmup)
    clocks = ClockSampler(dist.local)
    clocks.start()
    dist.barrier()
    t0 = time.time()
    sim.steps(DT, args.steps)
    wall = time.time() - t0
    st = sim.stats
    dev_s = dist.max(st.seconds)
    dist.barrier()
    clk = clocks.stop()
    per_rank = N * N * args.steps / dev_s
    value = per_rank * dist.ws
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32" if prec == _lib.MIXED else "f64",
            "data": "synthetic (seeded Gaussian chi, mean 600 K, std 40 K, l=16 cells)",
            "config": bench_config(args, extrap, dist.ws),
            "clocks": clk, "gpu_launches": int(st.kernel_launches),
            "vcycles_per_step": st.vcycles / args.steps, "refinements_per_step": st.refinements / args.steps,
            "extra_vcycles_per_step": st.extra_vcycles / args.steps,
            "wall_ms_per_step": 1e3 * wall / args.steps}
    if dist.rank != 0:
        return None
    if args.skip_extras:
        line["inner_cycles"] = args.inner
        return line

    # FP64 GPU path and the mixed-vs-FP64 error from the same initial state
    if prec == _lib.MIXED:
        nsteps = args.fp64_steps or min(args.warmup + args.steps, 60)
        a = ShearSim(P, chi, precision=_lib.FP64, tol_mode=_lib.TOL_RELATIVE, tol=RTOL, extrapolate=extrap)
        b = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=RTOL, extrapolate=extrap,
                     inner_cycles=args.inner)
        a.steps(DT, nsteps)
        b.steps(DT, nsteps)
        from parity import group_errors
        err = group_errors(a.fields(), b.fields(), N)
        # the same warm-up and timed steps as the mixed run: the tgmg_predict
        # cycle count settles over tens of steps, so a shorter window would
        # charge FP64 for the predictor's start-up
        a2 = ShearSim(P, chi, precision=_lib.FP64, tol_mode=_lib.TOL_RELATIVE, tol=RTOL, extrapolate=extrap)
        a2.steps(DT, args.warmup)
        k64 = args.steps
        a2.steps(DT, k64)
        fp64_value = N * N * k64 / a2.stats.seconds
        line["fp64"] = {"value": fp64_value, "ms_per_step": 1e3 * a2.stats.seconds / k64,
                        "vcycles_per_step": a2.stats.vcycles / k64,
                        "extra_vcycles_per_step": a2.stats.extra_vcycles / k64, "steps": k64}
        line["speedup_mixed_vs_fp64"] = value / dist.ws / fp64_value
        line["rel_err_mixed_vs_fp64"] = {"steps": nsteps, **{k: float(v) for k, v in err.items()}}
        for h in (a, b, a2):
            h.close()

    # the explicit step (shear_sim::step_forward) on the same grid and state
    # shape, dt = dx^2/2 as the reference's solve with tmult = 0.5
    if prec == _lib.MIXED:
        d = ShearSim(P, chi, precision=_lib.FP64)
        ddt = 0.5 * (2.0 / N) ** 2
        d.step_forward(ddt, 3)
        kd = 50
        d.step_forward(ddt, kd)
        line["direct"] = {"value": N * N * kd / d.stats.seconds, "unit": METRIC,
                          "ms_per_step": 1e3 * d.stats.seconds / kd, "steps": kd, "dt": ddt,
                          "GBs": DIRECT_BYTES_PER_CELL * N * N / (d.stats.seconds / kd) / 1e9,
                          "api": "stzg_step_direct (explicit step)"}
        d.close()

    # roofline of the dominant kernels, timed in isolation on the library's stream
    peak, peak_kind = measured_peaks()
    nn = N * (N + 1)
    t_adv = sim.time_kernel(DT, 0, 10)
    rows = {"advect": (t_adv, ADVECT_BYTES_PER_CELL * N * N, 1.0),
            "source": (sim.time_kernel(DT, 8, 10), SOURCE_BYTES_PER_NODE * nn, 1.0)}
    if prec == _lib.MIXED:
        t_v32 = sim.time_kernel(DT, 4, 10)
        t_rff = sim.time_kernel(DT, 5, 10)
        # refinement-pass V-cycles plus the one after convergence
        vc = (st.vcycles + st.extra_vcycles) / args.steps
        rows["vcycle_fp32"] = (t_v32, VCYCLE32_BYTES_PER_NODE * nn, vc)
        rows["residual_ff"] = (t_rff, RESIDFF_BYTES_PER_NODE * nn, st.refinements / args.steps + 1)
    else:
        t_v64 = sim.time_kernel(DT, 3, 10)
        rows["vcycle_fp64"] = (t_v64, VCYCLE64_BYTES_PER_NODE * nn, (st.vcycles + st.extra_vcycles) / args.steps)
    shares = {k: t * c for k, (t, b, c) in rows.items()}
    dom = max(shares, key=shares.get)
    t, b, c = rows[dom]
    achieved = b / (t * 1e-3) / 1e9
    pkey = "mixed" if prec == _lib.MIXED else "fp64"
    traffic = NCU_TRAFFIC_2048.get(dom, NCU_TRAFFIC_2048.get(f"{dom}_{pkey}"))
    line["roofline"] = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_kind": peak_kind,
                        "traffic": traffic * (N / 2048.0) ** 2 if traffic else None,
                        "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one launch under ncu "
                                          "(cold caches), scaled by cells",
                        "ms_per_launch": t, "algorithmic_bytes": b,
                        "share_of_step": shares[dom] / (1e3 * dev_s / args.steps)}
    if dom == "advect" and prec == _lib.MIXED:
        line["roofline"]["note"] = ("issue-bound float-float ENO arithmetic (issue slots 67% active, FP64 pipe "
                                    "11%, DRAM 14% under ncu); its DRAM traffic equals the algorithmic bytes")
    elif dom == "advect":
        line["roofline"]["note"] = "FP64-pipe-bound (FP64 pipe 83% active under ncu); HBM is not the limit"

    line["kernels"] = {k: {"ms": t, "per_step": c, "GBs": b / (t * 1e-3) / 1e9} for k, (t, b, c) in rows.items()}
    if prec == _lib.MIXED:
        # the FP32 V-cycle with its coarse levels (<= 512 columns) and tail in
        # one cooperative persistent kernel, against the per-level launches the
        # run used (same arithmetic, bitwise equal results)
        sched = {"used": "persistent" if sim.mg_persistent else "per_level", "per_level_ms": t_v32}
        try:
            sim.mg_persistent = True
            sched["persistent_ms"] = sim.time_kernel(DT, 4, 20)
            sim.mg_persistent = False
        except _lib.StzgError as e:
            sched["persistent_ms"] = None
            sched["persistent_unavailable"] = str(e)
        line["mg_coarse_schedule"] = sched
    line["mg_hbm_gbs"] = line["kernels"].get("vcycle_fp32", line["kernels"].get("vcycle_fp64"))["GBs"]
    if prec == _lib.MIXED:
        # the two top-level streaming kernels alone (the V-cycle's largest
        # byte movers): 26 B per fine node each (z and b read, z written, a
        # quarter node of the child's b written or z read)
        top = {}
        for kid, name in ((6, "down"), (7, "up")):
            try:
                t = sim.time_kernel(DT, kid, 20)
            except _lib.StzgError:
                continue
            gbs = TOP_BYTES_PER_NODE * nn / (t * 1e-3) / 1e9
            top[name] = {"us": 1e3 * t, "GBs": gbs, "frac": gbs / peak}
        if top:
            line["mg_top_level"] = {**top, "bytes_per_launch": TOP_BYTES_PER_NODE * nn, "peak": peak,
                                    "peak_kind": peak_kind,
                                    "l2": "back-to-back launches, no flush: z and b (8 B each per node) fit in "
                                          "the 129 MB L2 at 2048^2, so these are warm-L2 figures"}

    # end to end through the C ABI with host buffers: upload the state, step,
    # download the state, every step; a fresh handle repeats the timed
    # region (same warm-up, same steps) so the number is comparable to value
    import torch
    sim.close()
    cells, nodes = N * (N + 2), N * (N + 1)
    up = [torch.empty(cells, dtype=torch.float64, pin_memory=True) for _ in range(5)]
    up += [torch.empty(nodes, dtype=torch.float64, pin_memory=True) for _ in range(2)]
    up += [torch.empty(2 * nodes, dtype=torch.float64, pin_memory=True)]
    down = up + [torch.empty(N * N, dtype=torch.float64, pin_memory=True)]
    up_p, down_p = [t.data_ptr() for t in up], [t.data_ptr() for t in down]

    def e2e_run(one_call):
        h = ShearSim(P, chi, precision=prec, tol_mode=_lib.TOL_RELATIVE, tol=RTOL, extrapolate=extrap,
                     inner_cycles=args.inner)
        h.steps(DT, args.warmup)
        h.download(down_p)
        t0 = time.time()
        for _ in range(args.steps):
            if one_call:
                h.step_host(DT, up_p, down_p)
            else:
                h.upload(up_p)
                h.steps(DT, 1)
                h.download(down_p)
        dt_s = time.time() - t0
        h.close()
        return N * N * args.steps / dt_s * dist.ws

    def e2e_c_field_run():
        # the reference's own layout: one array of c_field records (19 doubles
        # per point, rows -1..n) in ordinary host memory, converted to and from
        # the pinned upload buffers on the host cores every step
        from stz_gb300.shear_sim import C_FIELD_DOUBLES, c_field_pack, c_field_unpack
        up_np = [t.numpy() for t in up]
        down_np = [t.numpy() for t in down]
        rec = np.zeros(((N + 2) * N, C_FIELD_DOUBLES))
        h = ShearSim(P, chi, precision=prec, tol_mode=_lib.TOL_RELATIVE, tol=RTOL, extrapolate=extrap,
                     inner_cycles=args.inner)
        h.steps(DT, args.warmup)
        h.download(down_p)
        c_field_unpack(down_np, N, N, rec)
        t_pack = t_unpack = 0.0
        t0 = time.time()
        for _ in range(args.steps):
            a = time.time()
            c_field_pack(rec, N, N, up_np)
            b = time.time()
            h.step_host(DT, up_p, down_p)
            c = time.time()
            c_field_unpack(down_np, N, N, rec)
            t_pack += b - a
            t_unpack += time.time() - c
        dt_s = time.time() - t0
        h.close()
        return {"value": N * N * args.steps / dt_s * dist.ws, "unit": METRIC,
                "pack_ms_per_step": 1e3 * t_pack / args.steps, "unpack_ms_per_step": 1e3 * t_unpack / args.steps,
                "host_threads": os.cpu_count(),
                "api": "stzg_c_field_pack + stzg_step_qs_host + stzg_c_field_unpack on the reference's "
                       "c_field array (152 B per point, pageable host memory)"}

    if prec == _lib.MIXED and not args.skip_batch:
        line["batched"] = batched_leg(args)
    e2e_one = e2e_run(True)
    e2e_three = e2e_run(False)
    e2e_aos = e2e_c_field_run()
    h2d = sum(t.numel() * 8 for t in up)
    d2h = sum(t.numel() * 8 for t in down)
    line["e2e"] = {"value": e2e_one, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                   "steps": args.steps, "warmup": args.warmup,
                   "api": "stzg_step_qs_host (upload, step, download in one call; pinned host buffers)",
                   "three_calls": {"value": e2e_three, "api": "stzg_upload + stzg_step_qs + stzg_download"},
                   "c_field_layout": e2e_aos}

    if not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(P, chi, args.cpu_steps)
        # parity on the benchmark's own grid and chi, and on a plastic-active
        # start (walls at +-0.04, CFL 0.41 at 2048^2, so the stress keeps
        # loading past the yield stress)
        from stz_gb300.params import simple_shear
        line["rel_err_vs_oracle"] = {
            "metric": "max |GPU - oracle| per field group over the group's scale",
            "elastic": parity_vs_oracle(P, chi, 4, extrap),
            "plastic_active": {"start": "tau = 1.02 s_y in every cell, walls at +-0.04",
                               **parity_vs_oracle(simple_shear(N, u_bdry=0.04), chi, 3, extrap, plastic=True)}}
    return line


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return 0
        line = run_reference(args, Dist(1, 0, 0))
        print(json.dumps(line), flush=True)
        return 0
    dist = Dist(ws, rank, local)
    line = run_ours(args, dist)
    if line is not None:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
