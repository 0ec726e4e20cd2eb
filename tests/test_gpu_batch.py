"""Batches: many simulations in one CUDA graph with device-side step and
multigrid loops, against the same simulations stepped one by one."""
import numpy as np
import pytest

from parity import group_errors
from stz_gb300 import _lib
from stz_gb300.batch import Batch
from stz_gb300.params import plastic_shear, simple_shear
from stz_gb300.shear_sim import ShearSim, random_chi

pytestmark = pytest.mark.gpu


def _members(plastic):
    # plastic members: walls at 4, yield near t=0.7; dt=0.005 keeps the
    # advective CFL number below 0.6 on the 64-cell grid
    sizes = [16, 24, 32, 48, 64] if plastic else [32, 48, 64, 96, 128]
    ps, chis = [], []
    for k, N in enumerate(sizes):
        p = plastic_shear(N, u_bdry=4.0, c0=0.3 + 0.05 * k) if plastic else simple_shear(N, c0=0.3 + 0.05 * k)
        ps.append(p)
        chis.append(random_chi(N, N, 4, 600.0, 20.0 + 5 * k, p.TZ, 40 + k))
    return ps, chis


@pytest.mark.parametrize("precision", [_lib.MIXED, _lib.FP64])
@pytest.mark.parametrize("plastic", [False, True])
def test_batch_matches_individual_runs(precision, plastic):
    ps, chis = _members(plastic)
    steps, dt = (160, 0.005) if plastic else (25, 0.01)
    b = Batch(ps, chis, precision=precision, tol=1e-11)
    st = b.run(dt, steps)
    assert st.failed == 0 and st.steps == steps * len(ps)
    assert st.kernel_launches > st.graph_kernels
    for k, (p, chi) in enumerate(zip(ps, chis)):
        ref = ShearSim(p, chi, precision=precision, tol_mode=_lib.TOL_RELATIVE, tol=1e-11, extrapolate=True)
        ref.steps(dt, steps)
        got = b.sim(k)
        assert abs(got.time - ref.time) < 1e-12
        err = group_errors(ref.fields(), got.fields(), p.n)
        assert max(err.values()) < 1e-8, (k, err)
        if plastic:
            assert np.max(got.get("eps_pl")) > 0


def test_batch_runs_continue_and_autotune():
    ps, chis = _members(False)
    b = Batch(ps, chis, precision=_lib.MIXED, tol=1e-10)
    tuned = b.autotune(0.01, steps=3)
    assert set(tuned) == {(p.m, p.n) for p in ps}
    for v in tuned.values():
        assert v["inner"] in (2, 3, 4) and v["fuse"] in (0, 1)
    b.run(0.01, 10)
    b.run(0.01, 10)  # same graph relaunched: the device clock continues
    ref = ShearSim(ps[2], chis[2], precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-10, extrapolate=True)
    ref.steps(0.01, 20)
    assert abs(b.sim(2).time - ref.time) < 1e-12
    err = group_errors(ref.fields(), b.sim(2).fields(), ps[2].n)
    assert max(err.values()) < 1e-8, err


@pytest.mark.parametrize("precision", [_lib.MIXED, _lib.FP64])
def test_batch_config3_sizes_against_oracle(precision):
    """Members of the batched configuration's grid sizes (192, 256, 384 and
    512: odd periodic lines in the 192 and 384 hierarchies) with their own
    chi and STZ parameters, run together in one graph, each against the CPU
    oracle from the same state (both solved to a relative residual of 1e-12;
    gate 1e-10 FP64, 1e-8 mixed)."""
    from oracle.bind import OracleSim
    sizes = [192, 256, 384, 512]
    rng = np.random.default_rng(3)
    ps, chis = [], []
    for k, N in enumerate(sizes):
        p = simple_shear(N, c0=float(rng.uniform(0.2, 0.6)), chi_inf_K=float(rng.uniform(800, 1000)))
        ps.append(p)
        chis.append(random_chi(N, N, 4, 600.0, float(rng.uniform(10, 50)), p.TZ, 60 + k))
    steps, dt = 5, 0.01
    b = Batch(ps, chis, precision=precision, tol=1e-12)
    st = b.run(dt, steps)
    assert st.failed == 0 and st.steps == steps * len(ps)
    gate = 1e-10 if precision == _lib.FP64 else 1e-8
    for k, (p, chi) in enumerate(zip(ps, chis)):
        o = OracleSim(p, chi)
        o.set_tolerance(1, 1e-13)
        o.steps(dt, steps)
        err = group_errors(o.fields(), b.sim(k).fields(), p.n)
        assert max(err.values()) < gate, (sizes[k], err)
    b.close()
