"""The CPU oracle (oracle/stz_oracle.c) against golden vectors that the
reference's own shear_sim produced (tests/golden/make_golden.py):
step_forward_quasistatic, step_forward, the initial states of init_fields
and initialize_chi_bicubic, and l2_comparison."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle.bind import OracleSim
from parity import group_errors


def test_oracle_matches_reference_golden(golden):
    name, P, meta, ref = golden
    sim = OracleSim(P, ref["chi0"])
    sim.set_tolerance(0, meta["acc_mult"])
    cycles = sim.steps(meta["dt"], meta["steps"])
    got = sim.fields()
    err = group_errors(ref, got, P.n)
    # Tight cases: solver error ~1e-12; the default-tolerance case carries the
    # reference's own ~1e-9 solver error on the stress (coarse operators are
    # formed in a different summation order, so iterates differ by rounding).
    gate = 1e-10 if meta["acc_mult"] <= 10 else 1e-8
    assert max(err.values()) < gate, (name, err)
    # Same V-cycle schedule (zebra Gauss-Seidel and the adaptive predictor are
    # restated exactly); allow a couple of cycles of drift near thresholds.
    assert abs(cycles - meta["cycles"]) <= max(2, 0.01 * meta["cycles"]), (cycles, meta["cycles"])
    assert abs(sim.time - meta["time"]) == 0.0


def test_golden_plastic_cases_are_plastic(golden):
    name, P, meta, ref = golden
    if name.startswith("elastic"):
        assert np.max(ref["eps_pl"]) == 0.0
    elif name not in ("thermal_nonlinear16",):
        # plastic-active variants: a large share of cells yields by the end
        assert np.mean(ref["ddev"][1:-1] > 0) > 0.1 or np.max(ref["eps_pl"]) > 0


def test_oracle_direct_step_matches_reference_golden(golden_direct):
    """The explicit step (shear_sim::step_forward, shear_sim.cc:185-276) in
    the frame loop of shear_sim::solve: the restatement repeats the
    reference's arithmetic operation for operation."""
    name, P, meta, ref = golden_direct
    sim = OracleSim(P, ref["chi0"])
    steps = sim.advance_direct(meta["dt"], meta["target"])
    got = sim.fields()
    err = group_errors(ref, got, P.n)
    assert max(err.values()) < 1e-13, (name, err)
    scale = max(np.abs(ref["ddev"]).max(), 1e-300)
    assert np.abs(got["ddev"] - ref["ddev"]).max() <= 1e-13 * scale
    assert steps == meta["steps"] and sim.time == meta["time"]


INIT_FIELDS = ("u", "v", "p", "q", "s", "tau", "chi", "X", "Y", "ddev")


def oracle_initial_state(P, meta, ref):
    sim = OracleSim(P)
    setup = meta["setup"]
    if setup[0] == "init":
        sim.init_fields(*setup[1:])
    else:
        sim.chi_bicubic(ref["bicubic_arr"], setup[2], setup[3])
    return sim


@pytest.mark.parametrize("name", golden_names("init"))
def test_oracle_initial_states_match_reference(name):
    """shear_sim::init_fields (chi cases 0-2) and initialize_chi_bicubic:
    every field of the initial state equals the reference's to rounding (the
    bicubic chi on the cells; its ghost rows are defined here, extrapolated,
    and left as they were by the reference), and quasi-static steps from it
    follow the reference."""
    P, meta, ref = load_golden(name)
    sim = oracle_initial_state(P, meta, ref)
    got = sim.fields()
    for k in INIT_FIELDS:
        a, b = ref[k + "0"], got[k]
        if k == "chi" and meta["setup"][0] == "bicubic":
            a, b = a[1:-1], b[1:-1]
        assert np.abs(a - b).max() <= 1e-15 * max(np.abs(a).max(), 1.0), (name, k)
    sim.set_tolerance(0, meta["acc_mult"])
    cycles = sim.steps(meta["dt"], meta["steps"])
    err = group_errors(ref, sim.fields(), P.n)
    assert max(err.values()) < 1e-10, (name, err)
    assert abs(cycles - meta["cycles"]) <= max(2, 0.01 * meta["cycles"])


@pytest.mark.parametrize("name", golden_names("l2"))
def test_oracle_l2_comparison_matches_reference(name):
    """The restated l2_comparison (shear_sim.cc:460-502) on the oracle's own
    runs from the fixture's chi: the explicit and the quasi-static run, then
    their weighted L2 differences, against the reference's."""
    P, meta, ref = load_golden(name)
    d = OracleSim(P, ref["chi0"])
    q = OracleSim(P, ref["chi0"])
    q.set_tolerance(0, meta["acc_mult"])
    got = [d.l2_comparison(q)]
    t_prev = 0.0
    for t in meta["frames"]:
        d.advance_direct(meta["dt"], t)
        q.steps((t - t_prev) / meta["qs_steps"], meta["qs_steps"])
        t_prev = t
        got.append(d.l2_comparison(q))
    got = np.array(got)
    np.testing.assert_allclose(got, ref["l2"], rtol=1e-9, atol=1e-300)
    for prefix, sim in (("direct_", d), ("qs_", q)):
        err = group_errors({k[len(prefix):]: v for k, v in ref.items() if k.startswith(prefix)}, sim.fields(), P.n)
        assert max(err.values()) < 1e-10, (name, prefix, err)


@pytest.mark.parametrize("name", golden_names("coarse"))
def test_oracle_coarse_operators_match_reference(name):
    """The oracle's generic Galerkin product R A P against the coarse stencils
    the reference's generated rat() stores (tgmg_level::s, tgmg.in.cc:667-736),
    all nine blocks and the inverse centre, on every level."""
    P, meta, ref = load_golden(name)
    o = OracleSim(P, np.full((P.n, P.m), 600 / 21000.0))
    assert [list(x) for x in o.mg_levels(meta["dt"])] == meta["levels"]
    for k in range(len(meta["levels"])):
        a, b = o.mg_stencil(meta["dt"], k), ref[f"level{k}"]
        assert np.max(np.abs(a - b)) <= 1e-14 * np.max(np.abs(b)), (name, k)
