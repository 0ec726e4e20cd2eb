"""The explicit (direct) step, shear_sim::step_forward (shear_sim.cc:185-276),
on the GPU against the reference's golden fixtures and the oracle."""
import numpy as np
import pytest

from oracle.bind import OracleSim
from parity import group_errors
from stz_gb300 import _lib
from stz_gb300.params import plastic_shear, simple_shear
from stz_gb300.shear_sim import ShearSim, random_chi

pytestmark = pytest.mark.gpu

FIELDS = ("p", "q", "s", "tau", "chi", "X", "Y", "u", "v")


def test_direct_matches_reference_golden(golden_direct):
    name, P, meta, ref = golden_direct
    with ShearSim(P, ref["chi0"]) as sim:
        steps = sim.advance_direct(meta["dt"], meta["target"])
        got = sim.fields()
        assert steps == meta["steps"] and sim.time == meta["time"]
    err = group_errors(ref, got, P.n)
    assert max(err.values()) < 1e-10, (name, err)
    scale = max(np.abs(ref["ddev"]).max(), 1e-300)
    assert np.abs(got["ddev"][1:-1] - ref["ddev"][1:-1]).max() <= 1e-10 * scale


@pytest.mark.parametrize("N,M", [(48, 48), (64, 40)])
def test_direct_matches_oracle(N, M):
    P = plastic_shear(N, M, u_bdry=4.0, s_y=0.2, viscosity=0.01, chi_diff=1e-3, chi_len=0.03)
    chi = random_chi(N, M, 3, 600.0, 30.0, P.TZ, 21)
    dx = (P.bx - P.ax) / N
    dt = 0.5 * dx * dx
    o = OracleSim(P, chi)
    o.steps_direct(dt, 300)
    for prec in (_lib.FP64, _lib.MIXED):
        with ShearSim(P, chi, precision=prec) as sim:
            sim.step_forward(dt, 300)
            err = group_errors(o.fields(), sim.fields(), M)
            assert max(err.values()) < 1e-10, (prec, err)
            assert sim.stats.kernel_launches > 0
    assert np.abs(o.eps_pl).max() > 0, "plastic-active case"


def test_direct_then_quasistatic():
    """A run that switches from explicit to quasi-static steps: the GPU's
    solve starts from the current velocity (the reference's from its last
    solution), so the two agree to the solver tolerance."""
    N = 32
    P = plastic_shear(N, viscosity=0.02)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 22)
    dt = 0.5 * (2.0 / N) ** 2
    o = OracleSim(P, chi)
    o.set_tolerance(_lib.TOL_RELATIVE, 1e-13)
    o.steps_direct(dt, 100)
    o.steps(0.01, 20)
    with ShearSim(P, chi, tol_mode=_lib.TOL_RELATIVE, tol=1e-13) as sim:
        sim.step_forward(dt, 100)
        sim.steps(0.01, 20)
        err = group_errors(o.fields(), sim.fields(), N, fields=FIELDS)
    assert max(err.values()) < 1e-9, err


def test_solve_frames_land_on_frame_times():
    N = 32
    P = simple_shear(N, viscosity=0.05)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 23)
    times = []
    with ShearSim(P, chi) as sim:
        sim.solve(0.1, 4, tmult=0.5, frame_callback=lambda k, s: times.append(s.time))
    np.testing.assert_allclose(times, [0.025, 0.05, 0.075, 0.1], rtol=0, atol=1e-15)
    with ShearSim(P, chi) as sim:
        with pytest.raises(_lib.StzgError):
            sim.advance_direct(1e-4, 0.0)
