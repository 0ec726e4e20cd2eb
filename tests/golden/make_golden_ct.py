"""Regenerates the golden fixtures of the coord_transforms step from the
reference itself.

Run where the SURGroup/STZ tree is available (the tree oracle/build_ref.sh
resolves: STZ_REFERENCE_ROOT, else the recipe's default):

    python tests/golden/make_golden_ct.py

It builds oracle/_ref/libctref.so (oracle/build_ref.sh: the reference's
esim/coord_transforms/simple_shear sources with oracle/ref_ct_driver.cc), sets
up the driver's Vitreloy configuration (shear_coord_transform.cc:20-89) on a
small grid with shear_sim::init_fields, runs step_forward_quasistatic, and
stores the initial and final fields (rows 0..n), the time and the V-cycle
count as tests/golden/ct_*.npz; the tracer cases (ct_tracers_*.npz) add
shear_sim::initialize_tracers / update_tracers, the ctdirect_*.npz cases
run the explicit shear_sim::step_forward from an advanced quasi-static state,
the ct_bicubic_*.npz cases the driver's bicubic chi set-up, and the
ct_frames_*.npz cases the files of write_files (fields, strain, tracers).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.bind_ct import FIELDS, ReferenceCt  # noqa: E402
from stz_gb300.ct_sim import transform_shear  # noqa: E402

# name -> (m, n, y_prd, chi_case, tem_base, tem_delta, dt, steps, lead, extra params)
# dt: the driver's frame interval over its 5 steps (tf/600); past about 40
# steps on these grids the periodic case's solve stops converging in the
# reference (exit 1), so the runs end before.  Stress passes yield (plastic
# flow) in each case.  With y periodic the elasticity operator annihilates
# rigid translations and the reference's velocity keeps whatever translation
# its own Gauss-Seidel iterates leave, which then moves the fields; those
# fixtures record one step (`steps` = 1) from the state after `lead` steps,
# so that a solver of another ordering can be compared field by field.
CASES = {
    "ct_prd64x32": (64, 32, True, 0, 580.0, 220.0, 0.5 / 1e-3 / 600, 1, 39, {}),
    "ct_prd48x24_line": (48, 24, True, 1, 580.0, 220.0, 0.5 / 1e-3 / 600, 1, 37, {}),
    "ct_wall64x32": (64, 32, False, 0, 580.0, 220.0, 3e6 / 2e4 / 600, 60, 0, {}),
    "ct_prd32x32_nodiff": (32, 32, True, 2, 580.0, 220.0, 0.5 / 1e-3 / 600, 1, 39, {"chi_len": 0.0}),
    "ct_prd64x32_elastic": (64, 32, True, 0, 580.0, 220.0, 0.5 / 1e-3 / 600, 1, 12, {}),
}


def make(name, case):
    m, n, yp, cc, base, delta, dt, steps, lead, extra = case
    P = transform_shear(m, n, y_prd=yp, **extra)
    ref = ReferenceCt(P)
    ref.init_fields(cc, base, delta)
    ref.steps(dt, lead)
    time0 = ref.time
    init = ref.fields()
    ref.steps(dt, steps)
    final = ref.fields()
    out = {"init_" + k: v for k, v in init.items()}
    out.update({"final_" + k: v for k, v in final.items()})
    params = {k: getattr(P, k) for k, _ in P._fields_}
    meta = {"params": params, "chi_case": cc, "dt": dt, "steps": steps, "lead": lead, "time0": time0,
            "time": ref.time, "vcount": ref.vcount}
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    dev = np.sqrt(3 * final["q"] ** 2 + final["s"] ** 2 + final["tau"] ** 2)[:-1]
    print(name, "time", ref.time, "vcount", ref.vcount, "max dev", dev.max(), "ddev", np.abs(final["ddev"]).max())
    ref.close()


# Lagrangian tracers: name -> (m, n, y_prd, chi_case, tem_base, tem_delta, dt,
# steps between updates, updates, tracer grid mm x nn).  The reference map
# (X, Y, rows 0..n) and the time before each update_tracers are stored with
# the tracers after it, so that the tracer update can be checked on the
# reference's own fields.
TRACER_CASES = {
    "ct_tracers_wall64x32": (64, 32, False, 0, 580.0, 220.0, 3e6 / 2e4 / 600, 10, 3, 16, 8),
    "ct_tracers_prd64x32": (64, 32, True, 0, 580.0, 220.0, 0.5 / 1e-3 / 600, 15, 2, 12, 6),
}


def make_tracers(name, case):
    m, n, yp, cc, base, delta, dt, every, updates, mm, nn = case
    P = transform_shear(m, n, y_prd=yp)
    ref = ReferenceCt(P)
    ref.init_fields(cc, base, delta)
    # one step first: the reference allocates its solver's work arrays on
    # the first solve and reads some of them before writing; allocating the
    # tracers' interpolators first hands it recycled, nonzero memory
    ref.steps(dt, 1)
    ref.initialize_tracers(mm, nn)
    out = {"tracers0": ref.tracers()}
    times = [ref.time]
    for u in range(updates):
        ref.steps(dt, every)
        out["X_%d" % u] = ref.get("X")
        out["Y_%d" % u] = ref.get("Y")
        times.append(ref.time)
        ref.update_tracers()
        out["tracers_%d" % u] = ref.tracers()
    params = {k: getattr(P, k) for k, _ in P._fields_}
    meta = {"params": params, "chi_case": cc, "dt": dt, "every": every, "updates": updates, "mm": mm, "nn": nn,
            "times": times}
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    tr = out["tracers_%d" % (updates - 1)]
    print(name, "tracers", len(tr), "max displacement", np.abs(tr[:, 2:4] - tr[:, 0:2]).max())
    ref.close()


# The explicit step: name -> (m, n, y_prd, chi_case, tem_base, tem_delta,
# quasi-static dt, quasi-static lead steps, explicit dt, explicit steps).  The
# state after the lead (plastic flow with y periodic, elastic with walls) and
# the time are stored with the state after the explicit steps.
DIRECT_CASES = {
    "ctdirect_wall64x32": (64, 32, False, 0, 580.0, 220.0, 3e6 / 2e4 / 600, 20, 0.005, 100),
    "ctdirect_prd64x32": (64, 32, True, 0, 580.0, 220.0, 0.5 / 1e-3 / 600, 39, 0.005, 60),
}


def make_direct(name, case):
    m, n, yp, cc, base, delta, qdt, lead, dt, steps = case
    P = transform_shear(m, n, y_prd=yp)
    ref = ReferenceCt(P)
    ref.init_fields(cc, base, delta)
    ref.steps(qdt, lead)
    time0 = ref.time
    init = ref.fields()
    ref.step_forward(dt, steps)
    final = ref.fields()
    out = {"init_" + k: v for k, v in init.items()}
    out.update({"final_" + k: v for k, v in final.items()})
    params = {k: getattr(P, k) for k, _ in P._fields_}
    meta = {"params": params, "chi_case": cc, "dt": dt, "steps": steps, "lead": lead, "time0": time0,
            "time": ref.time}
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "time", ref.time, "max|s| change", np.abs(final["s"] - init["s"]).max(),
          "ddev", np.abs(final["ddev"]).max())
    ref.close()


# The driver program's set-up (shear_coord_transform.cc:93-101): init_fields,
# then chi from the bicubic interpolant of a 64 x 32 sample array (a 2 x 2
# block of ones in a field of zeros, scaled 550 K + 30 K), then quasi-static
# steps: name -> (m, n, y_prd, chi_case, tem_base, tem_delta, dt, steps,
# sample array shape, lo, sca).  The walled case uses a random sample array
# (its one-sided first and last sample rows matter there).
BICUBIC_CASES = {
    "ct_bicubic_prd64x32": (64, 32, True, 0, 580.0, 220.0, 0.5 / 1e-3 / 600, 0, (32, 64), 550.0, 30.0),
    "ct_bicubic_wall48x24": (48, 24, False, 0, 580.0, 220.0, 3e6 / 2e4 / 600, 20, (7, 9), 560.0, 40.0),
}


def bicubic_array(shape):
    nn, mm = shape
    if (nn, mm) == (32, 64):
        a = np.zeros((nn, mm))
        a[15:17, 31:33] = 1.0  # i > 30 && i < 33 && j > 14 && j < 17
        return a
    return np.random.default_rng(7).random((nn, mm))


def make_bicubic(name, case):
    m, n, yp, cc, base, delta, dt, steps, shape, lo, sca = case
    P = transform_shear(m, n, y_prd=yp)
    ref = ReferenceCt(P)
    ref.init_fields(cc, base, delta)
    arr = bicubic_array(shape)
    ref.chi_bicubic(arr, lo / P.TZ, sca / P.TZ)
    init = ref.fields()
    ref.steps(dt, steps)
    final = ref.fields()
    out = {"init_" + k: v for k, v in init.items()}
    out.update({"final_" + k: v for k, v in final.items()})
    out["bicubic_arr"] = arr
    params = {k: getattr(P, k) for k, _ in P._fields_}
    meta = {"params": params, "chi_case": cc, "tem_base": base, "tem_delta": delta, "dt": dt, "steps": steps,
            "lo": lo / P.TZ, "sca": sca / P.TZ, "time": ref.time, "vcount": ref.vcount}
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "chi range (K)", init["chi"].min() * P.TZ, init["chi"].max() * P.TZ, "time", ref.time)
    ref.close()


# Frames (shear_sim::write_files with every output flag, strain and tracers
# included) of a state after quasi-static steps, twice (the second after
# more steps, so update_tracers runs inside it): name -> (m, n, y_prd,
# chi_case, tem_base, tem_delta, dt, steps before each frame, tracer grid).
# The fields before each frame are stored with the files' bytes.
FRAME_CASES = {
    "ct_frames_wall64x32": (64, 32, False, 0, 580.0, 220.0, 3e6 / 2e4 / 600, 10, (16, 8)),
    "ct_frames_prd40x20": (40, 20, True, 1, 580.0, 220.0, 0.5 / 1e-3 / 600, 10, (10, 5)),
}
FRAME_FLAGS = 16383
FRAME_FILES = ["u", "v", "p", "q", "s", "tau", "chi", "tem", "dev", "X", "Y", "Exx", "Exy", "Eyy", "E_I", "E_II",
               "Edev", "tra", "teml"]


def make_frames(name, case):
    import tempfile
    m, n, yp, cc, base, delta, dt, steps, (tm, tn) = case
    P = transform_shear(m, n, y_prd=yp)
    ref = ReferenceCt(P)
    ref.init_fields(cc, base, delta)
    ref.steps(dt, 1)  # the solver's work arrays first (see make_tracers)
    ref.initialize_tracers(tm, tn)
    out = {}
    times = []
    with tempfile.TemporaryDirectory() as tmp:
        for k in range(2):
            ref.steps(dt, steps)
            for f, v in ref.fields().items():
                out[f"state{k}_{f}"] = v
            out[f"tracers{k}"] = ref.tracers()
            times.append(ref.time)
            ref.write_files(tmp, k, FRAME_FLAGS)
            for f in FRAME_FILES:
                with open(os.path.join(tmp, f"{f}.{k}"), "rb") as fh:
                    out[f"file{k}_{f}"] = np.frombuffer(fh.read(), dtype=np.uint8)
    out["tracers_after"] = ref.tracers()
    params = {k: getattr(P, k) for k, _ in P._fields_}
    meta = {"params": params, "chi_case": cc, "dt": dt, "steps": steps, "times": times, "fflags": FRAME_FLAGS,
            "tracer_grid": [tm, tn], "files": FRAME_FILES}
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "times", times, "tracers", len(out["tracers_after"]))
    ref.close()


# l2_comparison_transform: a sheared-frame run (lamb, still walls) and a
# physical-frame run (lamb = 0, walls at +-lamb) from init_fields(1), explicit
# steps to the same time, as the reference's shear_compare driver does:
# name -> (m, n, lamb, dt multiplier tmult, explicit steps)
L2T_CASES = {"ct_l2t_32x16": (32, 16, 1e-2, 0.5, 40)}


def make_l2t(name, case):
    m, n, lamb, tmult, steps = case
    Pt = transform_shear(m, n, y_prd=False, lamb=lamb, u_bdry=0.0)
    Pp = transform_shear(m, n, y_prd=False, lamb=0.0, u_bdry=lamb)
    t, p = ReferenceCt(Pt), ReferenceCt(Pp)
    t.init_fields(1, 600.0, 200.0)
    p.init_fields(1, 600.0, 200.0)
    dx = (Pt.bx - Pt.ax) / m
    dt = dx * dx * tmult
    t.step_forward(dt, steps)
    p.step_forward(dt, steps)
    out = {"trans_" + k: v for k, v in t.fields().items()}
    out.update({"phys_" + k: v for k, v in p.fields().items()})
    out["l2"] = t.l2_comparison_transform(p)
    meta = {"trans": {k: getattr(Pt, k) for k, _ in Pt._fields_}, "phys": {k: getattr(Pp, k) for k, _ in Pp._fields_},
            "time": t.time, "dt": dt, "steps": steps}
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "time", t.time, "l2", out["l2"])
    t.close()
    p.close()


def main(argv):
    names = argv[1:] or list(CASES) + list(TRACER_CASES) + list(DIRECT_CASES) + list(BICUBIC_CASES) + \
        list(FRAME_CASES) + list(L2T_CASES)
    if len(names) == 1 and names[0] in L2T_CASES:
        make_l2t(names[0], L2T_CASES[names[0]])
        return
    if len(names) == 1 and names[0] in FRAME_CASES:
        make_frames(names[0], FRAME_CASES[names[0]])
        return
    if len(names) == 1 and names[0] in BICUBIC_CASES:
        make_bicubic(names[0], BICUBIC_CASES[names[0]])
        return
    if len(names) == 1 and names[0] in TRACER_CASES:
        make_tracers(names[0], TRACER_CASES[names[0]])
        return
    if len(names) == 1 and names[0] in DIRECT_CASES:
        make_direct(names[0], DIRECT_CASES[names[0]])
        return
    if len(names) == 1:
        make(names[0], CASES[names[0]])
        return
    # one process per case: the reference reads never-written ghost values
    # (ddev) and fresh allocations, which are zero only in a fresh process
    import subprocess
    for name in names:
        subprocess.check_call([sys.executable, os.path.abspath(__file__), name])


if __name__ == "__main__":
    main(sys.argv)
