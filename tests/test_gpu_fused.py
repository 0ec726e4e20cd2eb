"""The fused single-precision tile kernels (top level, N >= 80) and the
single-block tail of small levels, against the FP64 colour-by-colour path
and the oracle."""
import numpy as np
import pytest

from oracle.bind import OracleSim
from parity import group_errors
from stz_gb300 import _lib
from stz_gb300.params import plastic_shear, simple_shear
from stz_gb300.shear_sim import ShearSim, random_chi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [80, 96, 160, 256])
def test_mixed_vs_fp64_fused_sizes(N):
    P = plastic_shear(N, u_bdry=1.0)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, N)
    a = ShearSim(P, chi, precision=_lib.FP64, tol_mode=_lib.TOL_RELATIVE, tol=1e-11)
    b = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-11)
    a.steps(0.01, 25)
    b.steps(0.01, 25)
    err = group_errors(a.fields(), b.fields(), N)
    assert max(err.values()) < 1e-8, err
    # the FP32 V-cycles contract like the FP64 ones: comparable cycle counts
    assert b.cycles <= 1.5 * a.cycles + 25, (b.cycles, a.cycles)


@pytest.mark.parametrize("N", [128, 192])
def test_mixed_against_oracle(N):
    P = simple_shear(N)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 3)
    g = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-12)
    g.steps(0.01, 12)
    o = OracleSim(P, chi)
    o.set_tolerance(1, 1e-13)
    o.steps(0.01, 12)
    err = group_errors(o.fields(), g.fields(), N)
    assert max(err.values()) < 1e-9, err


@pytest.mark.parametrize("inner", [1, 3, 5])
def test_inner_cycle_counts_converge(inner):
    N = 128
    P = simple_shear(N)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 9)
    a = ShearSim(P, chi, precision=_lib.FP64, tol_mode=_lib.TOL_RELATIVE, tol=1e-11)
    b = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-11, inner_cycles=inner)
    a.steps(0.01, 10)
    b.steps(0.01, 10)
    err = group_errors(a.fields(), b.fields(), N)
    assert max(err.values()) < 1e-8, err


@pytest.mark.parametrize("N,M", [(256, 100), (192, 130), (128, 60), (160, 255), (250, 90)])
def test_streaming_kernels_non_square(N, M):
    """Non-square grids through the streaming kernels: odd and even node
    counts in y (the last row of an even line injects into the last coarse
    row), odd periodic lines below 64 points (the single-block tail), strips
    that end inside the grid, and an even top line with an odd child (125:
    colour-by-colour kernels below a streaming top level).  (Odd top lines
    are rejected at creation: the two-colour top-level smoother needs an even
    periodic line.)"""
    P = plastic_shear(N, M, u_bdry=1.0)
    chi = random_chi(N, M, 4, 600.0, 30.0, P.TZ, N + M)
    a = ShearSim(P, chi, precision=_lib.FP64, tol_mode=_lib.TOL_RELATIVE, tol=1e-11)
    b = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-11)
    a.steps(0.01, 20)
    b.steps(0.01, 20)
    err = group_errors(a.fields(), b.fields(), M)
    assert max(err.values()) < 1e-8, err
    assert b.cycles <= 1.5 * a.cycles + 25, (b.cycles, a.cycles)


def test_streaming_against_oracle_non_square():
    N, M = 256, 100
    P = simple_shear(N, M)
    chi = random_chi(N, M, 4, 600.0, 30.0, P.TZ, 5)
    g = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-12)
    g.steps(0.01, 8)
    o = OracleSim(P, chi)
    o.set_tolerance(1, 1e-13)
    o.steps(0.01, 8)
    err = group_errors(o.fields(), g.fields(), M)
    assert max(err.values()) < 1e-9, err


def test_streaming_runs_are_deterministic():
    """The swept z goes through a separate array between the down and up
    kernels, so two runs from the same state agree bit for bit."""
    N = 256
    P = plastic_shear(N, u_bdry=1.0)
    chi = random_chi(N, N, 4, 600.0, 30.0, P.TZ, 77)
    runs = []
    for _ in range(2):
        s = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-11)
        s.steps(0.01, 10)
        runs.append(s.fields())
        s.close()
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k


@pytest.mark.parametrize("case", ["elastic256", "plastic128", "plastic_rect160x96", "plastic64_cfl06"])
def test_float_float_advection(case):
    """Mixed-precision handles advect, form the projection source and correct
    the stresses in float-float arithmetic on the FP64 state (the default,
    STZG_ADV_AUTO).  Against the same handle with FP64 advection
    (STZG_ADV_FP64) and against the oracle, the group-normalised error stays
    inside the mixed-precision gate (1e-8): an elastic run, plastic-active
    runs (ENO choices, upwind switches, the plastic law) and a run at CFL 0.64
    over 60 steps, where the reference-map increments are largest."""
    if case == "elastic256":
        P, steps = simple_shear(256), 60
    elif case == "plastic128":
        P, steps = plastic_shear(128, u_bdry=1.0), 40
    elif case == "plastic64_cfl06":
        P, steps = plastic_shear(64, u_bdry=2.0), 60
    else:
        P, steps = plastic_shear(160, 96, u_bdry=1.0), 40
    N, M = P.m, P.n
    chi = random_chi(N, M, 4, 600.0, 30.0, P.TZ, 21)
    sp = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-12)
    dp = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-12, advection=_lib.ADV_FP64)
    sp.steps(0.01, steps)
    dp.steps(0.01, steps)
    err = group_errors(dp.fields(), sp.fields(), M)
    assert max(err.values()) < 1e-8, err
    o = OracleSim(P, chi)
    o.set_tolerance(1, 1e-13)
    o.steps(0.01, steps)
    err = group_errors(o.fields(), sp.fields(), M)
    assert max(err.values()) < 1e-8, err
