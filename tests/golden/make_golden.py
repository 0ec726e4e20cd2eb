"""Regenerates the golden fixtures from the reference itself.

Run in a checkout that has the SURGroup/STZ tree available (the tree
oracle/build_ref.sh resolves: STZ_REFERENCE_ROOT, else the recipe's default):

    python tests/golden/make_golden.py

It builds oracle/_ref/libstzref.so from the reference sources
(oracle/build_ref.sh), runs the reference's own
shear_sim::step_forward_quasistatic (esim/sb/main/shear_sim.cc:280) and
shear_sim::step_forward (shear_sim.cc:185) and the frame export and
diagnostics (output, qs_measure, tractions, compute_strain), the initial
states of init_fields and initialize_chi_bicubic and l2_comparison on seeded
inputs, and stores
inputs and outputs as compressed .npz files next to this script.  Names given
on the command line restrict it to those fixtures.  The chi inputs come from the oracle's seeded random-field generator;
they are stored in the fixture, so the fixtures do not depend on it.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.bind import ReferenceSim, random_chi  # noqa: E402
from stz_gb300.params import (STZ_LINEAR, STZ_NONLINEAR, STZ_NONLINEAR_ATHERMAL,  # noqa: E402
                              plastic_shear, simple_shear)

# name -> (params, chi (l, std, seed), dt, steps, tolerance multiplier)
# The tight cases use multiplier 10 in place of the default 1e4
# (qs_multi.cc:14): ~1e-12 solver error relative to the O(1) stresses of the
# plastic cases, inside a 1e-10 parity gate.  The elastic case's stresses are
# ~1e-5, so it needs multiplier 0.01 for the same relative accuracy.
# The thermal laws are stiff at t_scale=1 (the adaptive sub-stepping of
# shear_sim.cc:523-542 then never ends), so their cases use small t_scale.
CASES = {
    "elastic16_default": (simple_shear(16), (4, 30, 1), 0.01, 50, 1e4),
    "elastic32_tight": (simple_shear(32), (4, 30, 2), 0.01, 40, 0.01),
    "plastic32": (plastic_shear(32), (4, 30, 3), 0.01, 100, 10.0),
    "plastic24_oddlevels": (plastic_shear(24), (4, 30, 4), 0.01, 100, 10.0),
    "plastic_rect40x24": (plastic_shear(40, 24, u_bdry=3.0), (3, 30, 5), 0.01, 100, 10.0),
    "thermal_linear32": (plastic_shear(32, stz_model=STZ_LINEAR, u_bdry=3.0, t_scale=1e-18),
                         (4, 30, 6), 0.01, 100, 10.0),
    "thermal_nonlinear16": (plastic_shear(16, stz_model=STZ_NONLINEAR, u_bdry=3.0), (2, 30, 7), 0.01, 100, 10.0),
    "athermal_nonlinear16": (plastic_shear(16, stz_model=STZ_NONLINEAR_ATHERMAL), (2, 30, 8), 0.01, 100, 10.0),
    "truncation1_16": (plastic_shear(16, t_model=1), (2, 30, 9), 0.01, 100, 10.0),
    "chi_diffusion32": (plastic_shear(32, chi_diff=2e-3, chi_len=0.05), (4, 30, 10), 0.01, 100, 10.0),
    "viscous20": (plastic_shear(20, viscosity=0.02), (2, 30, 11), 0.01, 80, 10.0),
}


# Explicit (direct) steps, shear_sim::step_forward (shear_sim.cc:185-276),
# through the frame loop of shear_sim::solve (shear_sim.cc:120-140) with
# dt = dx^2 * tmult up to the target time:
# name -> (params, chi (l, std, seed), tmult, target time)
DIRECT_CASES = {
    "direct_elastic32": (simple_shear(32, viscosity=0.05, chi_diff=1e-3, chi_len=0.02), (4, 30, 12), 0.5, 0.3),
    "direct_plastic24": (plastic_shear(24, u_bdry=1.0, viscosity=0.02), (3, 30, 13), 0.5, 0.4),
    "direct_rect40x24": (plastic_shear(40, 24, u_bdry=2.0, viscosity=0.01, chi_diff=5e-4), (3, 30, 14), 0.4,
                         0.25),
}


def make_direct(name, spec):
    P, (l, std, seed), tmult, target = spec
    chi = random_chi(P.m, P.n, l, 600.0, std, P.TZ, seed)
    sim = ReferenceSim(P, chi)
    dx = (P.bx - P.ax) / P.m
    dt = dx * dx * tmult
    nsteps = sim.advance_direct(dt, target)
    f = sim.fields()
    out = {k: v for k, v in f.items()}
    out["chi0"] = chi
    meta = {"kind": "direct", "params": P.as_dict(), "dt": dt, "tmult": tmult, "target": target,
            "steps": int(nsteps), "time": sim.time,
            "source": "reference shear_sim::step_forward in the frame loop of shear_sim::solve, built from source"}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **out)
    return nsteps


# Frame export and diagnostics (shear_sim::output, qs_measure, tractions,
# compute_strain) on the state of a quasi-static run:
# name -> (params, chi (l, std, seed), dt, steps, tolerance multiplier)
FRAME_CASES = {
    "frames_plastic24": (plastic_shear(24), (3, 30, 15), 0.01, 90, 10.0),
}


def make_frames(name, spec):
    import tempfile
    P, (l, std, seed), dt, steps, mult = spec
    chi = random_chi(P.m, P.n, l, 600.0, std, P.TZ, seed)
    sim = ReferenceSim(P, chi)
    sim.set_acc_mult(mult)
    sim.steps(dt, steps)
    out = {k: v for k, v in sim.fields().items()}
    out["chi0"] = chi
    with tempfile.TemporaryDirectory() as tmp:
        for mode in range(11):
            out[f"output{mode}"] = sim.output(mode, tmp)
        sim.clear_cu()
        q, mx = sim.qs_measure(False)
        out["output11"] = sim.output(11, tmp)
        qs_stag = sim.qs_measure(True)
    out["qs"] = np.array([q, mx])
    out["qs_staggered"] = np.array(qs_stag)
    out["tractions"] = sim.tractions()
    out["strain"] = sim.compute_strain()
    meta = {"kind": "frames", "params": P.as_dict(), "dt": dt, "steps": steps, "acc_mult": mult, "time": sim.time,
            "source": "reference shear_sim::output, qs_measure, tractions, compute_strain after "
                      "step_forward_quasistatic, built from source"}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **out)


def make(name, spec):
    P, (l, std, seed), dt, steps, mult = spec
    chi = random_chi(P.m, P.n, l, 600.0, std, P.TZ, seed)
    sim = ReferenceSim(P, chi)
    sim.set_acc_mult(mult)
    cycles = sim.steps(dt, steps)
    f = sim.fields()
    out = {k: v for k, v in f.items()}
    out["chi0"] = chi
    out["vel"] = sim.vel()
    meta = {"params": P.as_dict(), "dt": dt, "steps": steps, "acc_mult": mult,
            "cycles": int(cycles), "time": sim.time,
            "source": "reference shear_sim::step_forward_quasistatic, built from source"}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **out)
    return cycles


# Initial states of the reference drivers, then quasi-static steps from
# them: shear_sim::init_fields (shear_sim.cc:60-114, chi cases 0-2) and
# shear_sim::initialize_chi_bicubic (shear_sim.cc:832-909):
# name -> (params, set-up, dt, steps, tolerance multiplier); set-up is
# ("init", chi_case, tem_base, tem_delta) or ("bicubic", (mm, nn, seed), lo, sca)
INIT_CASES = {
    "init_case0_32x24": (plastic_shear(32, 24, u_bdry=2.0), ("init", 0, 600.0, 200.0), 0.01, 40, 10.0),
    "init_case1_40x20": (plastic_shear(40, 20, u_bdry=2.0), ("init", 1, 630.0, 170.0), 0.01, 40, 10.0),
    "init_case2_48x24": (plastic_shear(48, 24, u_bdry=2.0, x_half=2.0), ("init", 2, 600.0, 200.0), 0.01, 40,
                         10.0),
    "bicubic_36x28": (plastic_shear(36, 28, u_bdry=2.0), ("bicubic", (9, 7, 21), 550.0 / 21000, 100.0 / 21000),
                      0.01, 40, 10.0),
}


def init_state(sim, setup):
    if setup[0] == "init":
        _, case, base, delta = setup
        sim.init_fields(case, base, delta)
        return {}
    _, (mm, nn, seed), lo, sca = setup
    arr = np.random.default_rng(seed).random((nn, mm))
    sim.chi_bicubic(arr, lo, sca)
    return {"bicubic_arr": arr}


def make_init(name, spec):
    P, setup, dt, steps, mult = spec
    sim = ReferenceSim(P)
    out = init_state(sim, setup)
    out.update({k + "0": v for k, v in sim.fields().items() if k != "eps_pl"})
    sim.set_acc_mult(mult)
    cycles = sim.steps(dt, steps)
    out.update(sim.fields())
    meta = {"kind": "init", "params": P.as_dict(), "setup": list(setup[:1]) + [setup[1] if setup[0] == "init"
                                                                              else list(setup[1])] +
            list(setup[2:]), "dt": dt, "steps": steps, "acc_mult": mult, "cycles": int(cycles), "time": sim.time,
            "source": "reference shear_sim::init_fields / initialize_chi_bicubic, then step_forward_quasistatic, "
                      "built from source"}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **out)
    return cycles


# shear_sim::l2_comparison (shear_sim.cc:460-502) of an explicit run and a
# quasi-static run from the same state, as the shear_compare driver does:
# name -> (params, chi (l, std, seed), tmult, frame times, quasi-static steps per frame, multiplier)
L2_CASES = {
    "l2cmp_32x16": (plastic_shear(32, 16, u_bdry=2.0, viscosity=0.02, x_half=2.0), (3, 30, 31), 0.5,
                           (0.05, 0.1, 0.15), 5, 10.0),
}


def make_l2(name, spec):
    P, (l, std, seed), tmult, frames, nq, mult = spec
    chi = random_chi(P.m, P.n, l, 600.0, std, P.TZ, seed)
    d = ReferenceSim(P, chi)
    q = ReferenceSim(P, chi)
    q.set_acc_mult(mult)
    dx = (P.bx - P.ax) / P.m
    dt = dx * dx * tmult
    out = {"chi0": chi}
    l2s = [d.l2_comparison(q)]
    t_prev = 0.0
    for k, t in enumerate(frames):
        d.advance_direct(dt, t)
        q.steps((t - t_prev) / nq, nq)
        t_prev = t
        l2s.append(d.l2_comparison(q))
    out["l2"] = np.array(l2s)
    out.update({"direct_" + k: v for k, v in d.fields().items()})
    out.update({"qs_" + k: v for k, v in q.fields().items()})
    meta = {"kind": "l2", "params": P.as_dict(), "tmult": tmult, "dt": dt, "frames": list(frames), "qs_steps": nq,
            "acc_mult": mult, "time": d.time,
            "source": "reference shear_sim::l2_comparison of a step_forward run and a step_forward_quasistatic "
                      "run, built from source"}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **out)
    return out["l2"][-1]


# Coarse Galerkin operators of the quasi-static system (tgmg::setup ->
# calculate_rat, tgmg.in.cc:667-736, generated compute_rat): every level's
# stored stencils (9 blocks and the inverse centre) for a grid shape.
COARSE_CASES = {"coarseops_24x24": (24, 24), "coarseops_32x32": (32, 32), "coarseops_40x72": (40, 72),
                "coarseops_80x80": (80, 80)}


def make_coarse(name, shape):
    m, n = shape
    P = simple_shear(m, n)
    sim = ReferenceSim(P, np.full((n, m), 600 / 21000.0))
    levels = sim.mg_levels(0.01)
    out = {f"level{k}": sim.mg_stencil(0.01, k) for k in range(len(levels))}
    meta = {"kind": "coarse", "params": P.as_dict(), "dt": 0.01, "levels": [list(x) for x in levels],
            "source": "reference tgmg_level::s after tgmg::setup of qs_multi, built from source"}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **out)
    return len(levels)


def main():
    only = sys.argv[1:]
    for name, shape in COARSE_CASES.items():
        if only and name not in only:
            continue
        print(f"{name}: {make_coarse(name, shape)} coarse levels")
    for name, spec in INIT_CASES.items():
        if only and name not in only:
            continue
        c = make_init(name, spec)
        print(f"{name}: {c} V-cycles")
    for name, spec in L2_CASES.items():
        if only and name not in only:
            continue
        l2 = make_l2(name, spec)
        print(f"{name}: l2 {l2}")
    for name, spec in CASES.items():
        if only and name not in only:
            continue
        c = make(name, spec)
        print(f"{name}: {c} V-cycles")
    for name, spec in FRAME_CASES.items():
        if only and name not in only:
            continue
        make_frames(name, spec)
        print(f"{name}: frames and diagnostics")
    for name, spec in DIRECT_CASES.items():
        if only and name not in only:
            continue
        k = make_direct(name, spec)
        print(f"{name}: {k} explicit steps")


if __name__ == "__main__":
    main()
