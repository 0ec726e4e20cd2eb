"""The benchmark configurations against the CPU oracle.

Configuration 0 (128x128, 200 steps, chi std 30 K, correlation length 4
cells), a bounded run of configuration 1 (1024x1024, chi l = 8 cells), the
headline configuration 2 (2048x2048, chi std 40 K, l = 16 cells) for a few
steps, and plastic-active variants of them: the stress starts just above the
yield stress everywhere (tau = 1.02 s_y) and the walls move fast enough
(CFL ~0.3-0.4) to keep loading it, so cells run the adaptive plastic
sub-stepping (shear_sim.cc:513-548) in every step and the plastic-strain
group is not vacuous.

FP64 is gated at 1e-10 (group-normalised), mixed precision at 1e-8.  Both
sides solve to a relative residual of 1e-13 (mixed: 1e-12, above the
float-float residual's floor): the stresses are differences of the solved
velocities over one cell, so a looser solve moves them by far more than the
gate in any implementation (the oracle against itself, 512x512, 5 steps:
stress 4e-8 at a relative residual of 1e-10, 5e-10 at 1e-12, 2.5e-12 at
1e-13).
"""
import numpy as np
import pytest

from oracle.bind import OracleSim
from parity import group_errors
from stz_gb300 import _lib
from stz_gb300.params import simple_shear
from stz_gb300.shear_sim import ShearSim, random_chi

pytestmark = pytest.mark.gpu

DT = 1e-2
FP64_GATE = 1e-10
MIXED_GATE = 1e-8


def prestress(sim, tau=1.02):
    """Uniform shear stress tau (units of the yield stress) in every cell,
    ghost rows included."""
    t = sim.get("tau")
    t[:] = tau
    sim.set("tau", t)


def oracle_run(P, chi, nsteps, tol, plastic=False):
    o = OracleSim(P, chi)
    o.set_tolerance(1, tol)
    if plastic:
        prestress(o)
    o.steps(DT, nsteps)
    return o.fields()


def gpu_run(P, chi, nsteps, precision, tol, plastic=False, extrapolate=1):
    g = ShearSim(P, chi, precision=precision, tol_mode=_lib.TOL_RELATIVE, tol=tol, extrapolate=extrapolate)
    if plastic:
        prestress(g)
    g.steps(DT, nsteps)
    f = g.fields()
    g.close()
    return f


def check(ref, P, chi, nsteps, tol_fp64=1e-13, tol_mixed=1e-12, plastic=False):
    N = P.n
    e64 = group_errors(ref, gpu_run(P, chi, nsteps, _lib.FP64, tol_fp64, plastic), N)
    assert max(e64.values()) < FP64_GATE, e64
    emx = group_errors(ref, gpu_run(P, chi, nsteps, _lib.MIXED, tol_mixed, plastic), N)
    assert max(emx.values()) < MIXED_GATE, emx
    return e64, emx


def test_config0_128_200_steps():
    """Configuration 0: 128x128, 200 steps of dt = 1e-2."""
    N = 128
    P = simple_shear(N)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 11)
    ref = oracle_run(P, chi, 200, 1e-13)
    check(ref, P, chi, 200)


def test_config0_plastic_active():
    N = 128
    P = simple_shear(N, u_bdry=0.5)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 12)
    o = OracleSim(P, chi)
    o.set_tolerance(1, 1e-13)
    prestress(o)
    o.steps(DT, 49)
    e0 = o.eps_pl.copy()
    o.steps(DT, 1)
    ref = o.fields()
    # yielding in the last step too, not only in the first
    assert (ref["eps_pl"].ravel() > e0).mean() > 0.2
    check(ref, P, chi, 50, plastic=True)


def test_config1_1024_bounded():
    """Configuration 1 (1024x1024, chi l = 8 cells), 10 steps."""
    N = 1024
    P = simple_shear(N)
    chi = random_chi(N, N, 8, 600.0, 30.0, P.TZ, 13)
    ref = oracle_run(P, chi, 10, 1e-13)
    check(ref, P, chi, 10)


@pytest.mark.parametrize("plastic", [False, True])
def test_config2_2048_headline(plastic):
    """Configuration 2 (2048x2048, chi std 40 K, l = 16 cells), 4 steps, and
    its plastic-active variant."""
    N = 2048
    P = simple_shear(N, u_bdry=0.04 if plastic else 1e-4)
    chi = random_chi(N, N, 16, 600.0, 40.0, P.TZ, 2)
    ref = oracle_run(P, chi, 4, 1e-13, plastic=plastic)
    if plastic:
        assert ref["eps_pl"].max() > 1e-3
    check(ref, P, chi, 4, plastic=plastic)


def test_device_loop_stops_at_the_tolerance():
    """The relative-tolerance solve ends on the device as soon as the
    residual meets the tolerance: each solve's final relative residual is at
    most tol, and a looser tolerance never needs more V-cycles."""
    N = 256
    P = simple_shear(N)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 14)
    counts = {}
    for prec in (_lib.FP64, _lib.MIXED):
        for tol in (1e-6, 1e-10):
            g = ShearSim(P, chi, precision=prec, tol_mode=_lib.TOL_RELATIVE, tol=tol, extrapolate=1)
            g.steps(DT, 5)
            st = g.stats
            assert st.last_error <= tol, (prec, tol, st.last_error)
            counts[prec, tol] = st.vcycles
            g.close()
        assert counts[prec, 1e-6] <= counts[prec, 1e-10], counts
