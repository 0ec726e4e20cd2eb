"""Regenerates the golden fixtures from the reference itself.

Run in a checkout that has the SURGroup/STZ tree available (default
/root/reference, override with STZ_REFERENCE_ROOT):

    python tests/golden/make_golden.py

It builds oracle/_ref/libstzref.so from the reference sources
(oracle/build_ref.sh), runs the reference's own
shear_sim::step_forward_quasistatic (esim/sb/main/shear_sim.cc:280) and
shear_sim::step_forward (shear_sim.cc:185) and the frame export and
diagnostics (output, qs_measure, tractions, compute_strain) on seeded
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


def main():
    only = sys.argv[1:]
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
