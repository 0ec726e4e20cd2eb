"""Parity of the coord_transforms step on the GPU (include/stzg_ct.h) with
the reference's own esim/coord_transforms/simple_shear shear_sim (golden
fixtures): from the reference's fields, the same quasi-static steps (60 steps
with walls; one step from advanced states with y periodic, where the
velocity is defined up to a translation; chi diffusion on and off, three chi
set-ups, elastic and plastic) give the same fields."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_names

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "p", "q", "s", "tau", "chi", "X", "Y", "ddev")


def _load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return json.loads(str(d["meta"])), {k: d[k] for k in d.files if k != "meta"}


def _params(meta):
    from stz_gb300.ct_sim import CtParams
    P = CtParams()
    for k, v in meta["params"].items():
        setattr(P, k, v)
    return P


def ct_errors(ref, got, P):
    """Group-normalised max errors over rows 0..n-1 (cells) and 0..n (nodes).
    With y periodic the velocity is defined up to a rigid translation (the
    operator's null space), so it is compared with its mean removed."""
    n = P.n
    cells = slice(0, n)
    dev = np.sqrt(3 * ref["q"] ** 2 + ref["s"] ** 2 + ref["tau"] ** 2)[cells]
    s_scale = max(np.abs(ref["p"][cells]).max() + dev.max(), 1e-300)
    out = {"stress": max(np.abs(got[k][cells] - ref[k][cells]).max() for k in ("p", "q", "s", "tau")) / s_scale,
           "chi": np.abs(got["chi"][cells] - ref["chi"][cells]).max() / np.abs(ref["chi"][cells]).max(),
           "refmap": max(np.abs(got["X"] - ref["X"]).max() / (P.bx - P.ax),
                         np.abs(got["Y"] - ref["Y"]).max() / (P.by - P.ay))}
    vscale = max(np.abs(ref["u"]).max(), np.abs(ref["v"]).max(), 1e-300)
    du, dv = got["u"] - ref["u"], got["v"] - ref["v"]
    if P.y_prd:
        du, dv = du[:n] - du[:n].mean(), dv[:n] - dv[:n].mean()
    out["velocity"] = max(np.abs(du).max(), np.abs(dv).max()) / vscale
    dscale = np.abs(ref["ddev"][cells]).max()
    out["ddev"] = np.abs(got["ddev"][cells] - ref["ddev"][cells]).max() / dscale if dscale > 0 else 0.0
    return out


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("name", golden_names("ct"))
def test_ct_steps_match_reference(name, mixed):
    """Also with the projection solved in mixed precision (FP32 V-cycles
    inside FP64 refinement, the same threshold on the FP64 residual), under
    the same gates."""
    from stz_gb300.ct_sim import CtSim
    meta, arr = _load(name)
    P = _params(meta)
    sim = CtSim(P)
    if mixed:
        sim.set_precision(True)
    sim.time = meta["time0"]
    for k in FIELDS:
        sim.set(k, arr["init_" + k])
    sim.step_forward_quasistatic(meta["dt"], meta["steps"])
    assert sim.time == pytest.approx(meta["time"], rel=1e-14)
    got = sim.fields()
    ref = {k: arr["final_" + k] for k in FIELDS}
    err = ct_errors(ref, got, P)
    # both solves stop at the reference's threshold on the mean squared
    # residual of the preconditioned system, acc = (DBL_EPSILON*1e4*2)^2
    # (qs_multi.cc:11): a residual of sqrt(acc) ~ 4e-12 per node over the
    # smallest nonzero eigenvalue of the operator (~1e-2 on these periodic
    # grids) leaves each solver a velocity error up to ~1e-5 of its scale;
    # the stresses take velocity gradients times dt and agree far closer
    vel = err.pop("velocity")
    assert vel < 1e-5, (vel, err)
    assert max(err.values()) < 1e-7, err
    if "elastic" not in name:
        assert np.abs(ref["ddev"]).max() > 0  # the case reached plastic flow
    sim.close()


def test_ct_init_fields_match_reference():
    """shear_sim::init_fields on the GPU handle reproduces the reference's
    initial state (chi cases 0-2, periodic and walled)."""
    from stz_gb300.ct_sim import CtSim
    for name in golden_names("ct"):
        meta, arr = _load(name)
        if meta["lead"]:
            continue
        P = _params(meta)
        sim = CtSim(P)
        sim.init_fields(meta["chi_case"], 580.0, 220.0)
        for k in FIELDS:
            assert np.allclose(sim.get(k), arr["init_" + k], rtol=1e-14, atol=1e-15), (name, k)
        sim.close()


@pytest.mark.parametrize("name", golden_names("ct_tracers"))
def test_ct_tracers_match_reference(name):
    """initialize_tracers / update_tracers on the reference's own reference
    map (set before each update at the reference's time): the same tracer
    positions (Newton on the bicubic interpolant) and velocity estimates."""
    from stz_gb300.ct_sim import CtSim
    meta, d = _load(name)
    P = _params(meta)
    g = CtSim(P)
    times = meta["times"]
    g.time = times[0]
    g.initialize_tracers(meta["mm"], meta["nn"])
    assert np.array_equal(g.tracers(), d["tracers0"])
    L = max(P.bx - P.ax, P.by - P.ay)
    for u in range(meta["updates"]):
        g.time = times[u + 1]
        g.set("X", d["X_%d" % u])
        g.set("Y", d["Y_%d" % u])
        assert g.update_tracers() == 0
        got, ref = g.tracers(), d["tracers_%d" % u]
        assert got.shape == ref.shape
        assert np.abs(got[:, :4] - ref[:, :4]).max() < 1e-12 * L, np.abs(got[:, :4] - ref[:, :4]).max()
        vscale = max(np.abs(ref[:, 4:]).max(), 1e-300)
        assert np.abs(got[:, 4:] - ref[:, 4:]).max() < 1e-9 * vscale
    g.close()


@pytest.mark.parametrize("name", golden_names("ct_direct"))
def test_ct_explicit_step_matches_reference(name):
    """shear_sim::step_forward (the explicit step) from the reference's own
    advanced state: the same fields after 60-100 steps (no solver, so the
    only differences are roundings)."""
    from stz_gb300.ct_sim import CtSim
    meta, arr = _load(name)
    P = _params(meta)
    sim = CtSim(P)
    sim.time = meta["time0"]
    for k in FIELDS:
        sim.set(k, arr["init_" + k])
    sim.step_forward(meta["dt"], meta["steps"])
    assert sim.time == pytest.approx(meta["time"], rel=1e-14)
    ref = {k: arr["final_" + k] for k in FIELDS}
    got = sim.fields()
    err = ct_errors(ref, got, P)
    assert max(err.values()) < 1e-10, err
    # the update moved the state
    assert np.abs(ref["s"] - arr["init_s"]).max() > 1e-4
    sim.close()


@pytest.mark.parametrize("name", golden_names("ct_bicubic"))
def test_ct_chi_bicubic_matches_reference(name):
    """shear_sim::initialize_chi_bicubic of the variant (the driver program's
    set-up: init_fields, then chi from a sample array) reproduces the
    reference's state, ghost layers through set_boundaries included; with
    walls, quasi-static steps from it follow the reference."""
    from stz_gb300.ct_sim import CtSim
    meta, arr = _load(name)
    P = _params(meta)
    sim = CtSim(P)
    sim.init_fields(meta["chi_case"], meta["tem_base"], meta["tem_delta"])
    sim.initialize_chi_bicubic(arr["bicubic_arr"], meta["lo"], meta["sca"])
    for k in FIELDS:
        a, b = sim.get(k), arr["init_" + k]
        assert np.abs(a - b).max() <= 1e-15 * max(np.abs(b).max(), 1.0), (name, k)
    if meta["steps"]:
        sim.step_forward_quasistatic(meta["dt"], meta["steps"])
        err = ct_errors({k: arr["final_" + k] for k in FIELDS}, sim.fields(), P)
        vel = err.pop("velocity")
        assert vel < 1e-5, (vel, err)
        assert max(err.values()) < 1e-7, err
    sim.close()


@pytest.mark.parametrize("name", golden_names("ct_frames"))
def test_ct_frames_match_reference(name, tmp_path):
    """shear_sim::write_files of the variant with every output flag: from the
    reference's own state, the field files equal the reference's byte for
    byte, the strain files (compute_strain with set_strain_boundaries) and
    the tracer files (bicubic interpolation at the tracers; at frame 1 after
    the tracers' Newton update on the GPU) agree to float rounding."""
    from stz_gb300.ct_sim import CtSim
    meta, arr = _load(name)
    P = _params(meta)
    sim = CtSim(P)
    sim.time = meta["times"][0]
    tm, tn = meta["tracer_grid"]
    sim.initialize_tracers(tm, tn)
    field_files = ["u", "v", "p", "q", "s", "tau", "chi", "tem", "dev", "X", "Y"]
    for k in range(2):
        sim.time = meta["times"][k]  # set_field applies the wall positions of the current time
        for f in FIELDS:
            sim.set(f, arr[f"state{k}_{f}"])
        sim.write_files(tmp_path, k, meta["fflags"])
        for f in meta["files"]:
            got = (tmp_path / f"{f}.{k}").read_bytes()
            ref = arr[f"file{k}_{f}"].tobytes()
            if f in field_files:
                assert got == ref, (k, f)
            elif f == "tra":
                a = np.loadtxt(tmp_path / f"tra.{k}")
                b = np.array([[float(x) for x in ln.split()] for ln in ref.decode().splitlines()])
                assert a.shape == b.shape, (k, f)
                np.testing.assert_allclose(a, b, rtol=1e-8, atol=1e-10 * np.abs(b).max(), err_msg=f"{k} {f}")
            else:
                a, b = np.frombuffer(got, np.float32), np.frombuffer(ref, np.float32)
                assert a.shape == b.shape, (k, f)
                np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-6 * np.abs(b).max(), err_msg=f"{k} {f}")
    sim.close()


def test_ct_frame_loop_writes_frames(tmp_path):
    """stzg_ct_solve_quasistatic: frame 0, then the steps and files of every
    frame (the frame loop of shear_sim::solve_quasistatic)."""
    from stz_gb300.ct_sim import CtSim, transform_shear
    P = transform_shear(32, 16, y_prd=False)
    sim = CtSim(P)
    sim.init_fields(0, 580.0, 220.0)
    sim.solve_quasistatic(3 * 0.25, 3, 2, tmp_path, 4 | 256 | 2048)
    for k in range(4):
        for f in ("p", "dev", "Exx", "Exy", "Eyy"):
            assert (tmp_path / f"{f}.{k}").stat().st_size > 0
    assert sim.time == pytest.approx(0.75, rel=1e-14)
    sim.close()


@pytest.mark.parametrize("name", golden_names("ct_l2t"))
def test_ct_l2_comparison_transform_matches_reference(name):
    """shear_sim::l2_comparison_transform on handles holding the reference's
    sheared-frame and physical-frame states: the reference's four numbers to
    rounding, but for the top node row of the reference-map term.  The
    reference's extra line (shear_sim.cc:675) starts at fm + gmn, and gmn is
    gm*gn, the whole allocation (shear_sim.cc:30), so it reads past both grids;
    in the fixture's process that memory held zeros, which leaves u, v equal to
    row n's wall values here but drops row n's X, Y differences.  The handle
    sums row n itself, so l2[3] is the reference's value plus that row's
    0.5 (dX^2 + dY^2) dx dy, formed here from the fixture fields."""
    from stz_gb300.ct_sim import CtParams, CtSim
    meta, arr = _load(name)

    def handle(key, prefix):
        P = CtParams()
        for k, v in meta[key].items():
            setattr(P, k, v)
        h = CtSim(P)
        h.time = meta["time"]
        for f in FIELDS:
            h.set(f, arr[prefix + f])
        return h

    t, p = handle("trans", "trans_"), handle("phys", "phys_")
    P = t.P
    n = P.n
    top = 0.5 * ((arr["trans_X"][n] - arr["phys_X"][n]) ** 2 + (arr["trans_Y"][n] - arr["phys_Y"][n]) ** 2).sum()
    want = np.array(arr["l2"], dtype=float)
    want[3] += top * (P.bx - P.ax) / P.m * (P.by - P.ay) / n
    assert top > 0  # the case moves the physical walls: row n differs
    np.testing.assert_allclose(t.l2_comparison_transform(p), want, rtol=1e-12, atol=1e-300)
    t.close()
    p.close()


def test_ct_batch_matches_single_handles():
    """stzg_ct_batch_step_qs over handles of different sizes, boundary
    conditions and strain rates, from several host threads: every handle ends
    bit for bit where stzg_ct_step_qs alone takes it, with the same V-cycle
    counts."""
    from stz_gb300.ct_sim import CtSim, batch_step_qs, transform_shear
    cases = [(32, 16, True, 1e-3), (48, 32, False, 0.0), (64, 32, True, 2e-3), (40, 24, False, 0.0),
             (64, 64, True, 5e-4), (96, 48, False, 0.0)]

    def make():
        out = []
        for k, (m, n, yp, lamb) in enumerate(cases):
            sim = CtSim(transform_shear(m, n, y_prd=yp, lamb=lamb if yp else None))
            sim.init_fields(k % 3, 600.0 + 10 * k, 200.0)
            out.append(sim)
        return out

    dt, steps = 2e-3, 5
    solo = make()
    for s in solo:
        s.step_forward_quasistatic(dt, steps)
    batch = make()
    vc, sec = batch_step_qs(batch, dt, steps, threads=4)
    assert sec > 0
    for a, b, v in zip(solo, batch, vc):
        assert v == a.vcycles
        fa, fb = a.fields(), b.fields()
        for k in fa:
            assert np.array_equal(fa[k], fb[k]), k
        assert a.time == b.time
    for s in solo + batch:
        s.close()


@pytest.mark.parametrize("m,n,yp", [(96, 48, False), (128, 64, True)])
def test_ct_mixed_matches_fp64(m, n, yp):
    """The projection in mixed precision against FP64 over 25 steps from the
    driver program's set-up (walls; y periodic at the driver's strain rate):
    both stop at the reference's threshold on the FP64 residual, so the
    fields agree to the gates of the reference comparison, and a refinement
    pass contracts like an FP64 V-cycle (as many passes as V-cycles, give or
    take a few)."""
    from stz_gb300.ct_sim import CtSim, transform_shear
    P = transform_shear(m, n, y_prd=yp, lamb=1e-3 if yp else None)
    sims = []
    for mixed in (False, True):
        sim = CtSim(P)
        sim.init_fields(0, 580.0, 220.0)
        if mixed:
            sim.set_precision(True)
        # the driver program's dt: tf/600 of its duration
        sim.step_forward_quasistatic((0.5 / 1e-3 if yp else 3e6 / 2e4) / 600, 25)
        sims.append(sim)
    a, b = sims
    err = ct_errors(a.fields(), b.fields(), P)
    vel = err.pop("velocity")
    assert vel < 1e-5, (vel, err)
    assert max(err.values()) < 1e-7, err
    assert abs(b.vcycles - a.vcycles) <= max(3, a.vcycles // 5), (a.vcycles, b.vcycles)
    for s in sims:
        s.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_ct_checked_solve_policy(mixed):
    """The residual-checked solve against the reference's predictor over 25
    steps from the driver program's set-up (y periodic, 128x64): the same
    threshold, so the fields agree to the reference comparison's gates, with
    fewer V-cycles (the predictor starts at eight per solve)."""
    from stz_gb300.ct_sim import CtSim, transform_shear
    P = transform_shear(128, 64, y_prd=True, lamb=1e-3)
    sims = []
    for checked in (False, True):
        sim = CtSim(P)
        sim.init_fields(0, 580.0, 220.0)
        sim.set_precision(mixed)
        sim.set_solve_policy(checked)
        sim.step_forward_quasistatic(0.5 / 1e-3 / 600, 25)
        sims.append(sim)
    a, b = sims
    err = ct_errors(a.fields(), b.fields(), P)
    vel = err.pop("velocity")
    assert vel < 1e-5, (vel, err)
    assert max(err.values()) < 1e-7, err
    assert b.vcycles < a.vcycles, (a.vcycles, b.vcycles)
    for s in sims:
        s.close()


def test_ct_bad_settings_are_statuses():
    """Out-of-range precision and solve-policy values, and a null handle, are
    STZG_EINVAL (1), and the handle still steps."""
    from stz_gb300.ct_sim import CtSim, transform_shear
    sim = CtSim(transform_shear(32, 16))
    assert sim.lib.stzg_ct_set_precision(sim.h, 2) == 1
    assert sim.lib.stzg_ct_set_solve_policy(sim.h, 2) == 1
    assert sim.lib.stzg_ct_set_solve_policy(None, 1) == 1
    sim.init_fields(0, 580.0, 220.0)
    sim.step_forward_quasistatic(0.5 / 1e-3 / 600, 2)
    sim.close()
