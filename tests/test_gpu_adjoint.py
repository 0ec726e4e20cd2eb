"""Adjoint of the quasi-static step: gradients against central finite
differences of the GPU forward run and of the FP64 CPU oracle.

Case: adjoint_shear (plastic flow over the last ~30 of 100 steps), loss =
dx dy sum (eps_pl - target)^2 with the target from a forward run whose c0,
Omega*eps0, chi_inf and s_y are 5 % larger.  Tolerance: 1e-6 relative for
every parameter gradient and for directional derivatives in chi.
"""
import numpy as np
import pytest

from stz_gb300 import _lib
from stz_gb300.adjoint import PARAM_NAMES, PlasticStrainLoss, StepAdjoint, with_params
from stz_gb300.params import ADJOINT_DT, adjoint_shear
from stz_gb300.shear_sim import ShearSim, random_chi

pytestmark = pytest.mark.gpu

TOL = 1e-6
EINVAL = 1
SOLVER = dict(tol_mode=_lib.TOL_RELATIVE, tol=1e-13)


def make_case(N, steps, seed=11):
    P = adjoint_shear(N)
    chi = random_chi(N, N, 4.0, 600.0, 30.0, P.TZ, seed)
    theta = np.array([getattr(P, k) for k in PARAM_NAMES])
    with ShearSim(with_params(P, theta * 1.05), chi, **SOLVER) as sim:
        sim.steps(ADJOINT_DT, steps)
        target = sim.get("eps_pl")
    assert np.abs(target).max() > 1e-3, "the case must be plastic-active"
    return P, chi, theta, target


def gpu_loss(P, theta, chi, target, steps, **kw):
    with ShearSim(with_params(P, theta), chi, **SOLVER, **kw) as sim:
        return StepAdjoint(sim, ADJOINT_DT, steps, 10).forward(target)


def gpu_grad(P, theta, chi, target, steps, every=10, dloss=1.0, **kw):
    with ShearSim(with_params(P, theta), chi, **SOLVER, **kw) as sim:
        adj = StepAdjoint(sim, ADJOINT_DT, steps, every)
        L = adj.forward(target)
        gp, gc = adj.backward(dloss)
    return L, gp, gc


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def case64():
    return make_case(64, 100)


def test_parameter_gradients_vs_central_fd(case64):
    P, chi, theta, target = case64
    L, gp, _ = gpu_grad(P, theta, chi, target, 100)
    assert L > 0
    for k, name in enumerate(PARAM_NAMES):
        h = 1e-6 * abs(theta[k])
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (gpu_loss(P, tp, chi, target, 100) - gpu_loss(P, tm, chi, target, 100)) / (2 * h)
        assert abs(fd) > 0, name
        assert rel(gp[k], fd) < TOL, (name, gp[k], fd)


def test_chi_gradient_directional_fd(case64):
    """Directional derivatives in chi along a uniform shift, the chi anomaly
    and the lowest x and y modes, by central differences with step 1e-7
    (relative to max chi).  The loss is only piecewise smooth in chi: the
    ENO2 stencil choice (shear_sim.cc:653-655) compares two second
    differences, and a perturbation of chi at t = 0 flips a few of the
    ~10^7 choices of the run, each a jump of the discrete loss.  At step 1e-6
    the central differences along the x mode pick up such jumps (5e-5
    relative scatter between steps 1e-5 and 1e-6); at 1e-7 the adjoint and
    the differences agree to 1e-8 along these directions."""
    P, chi, theta, target = case64
    _, _, gc = gpu_grad(P, theta, chi, target, 100)
    assert np.abs(gc).max() > 0
    n, m = chi.shape
    jj, ii = np.mgrid[0:n, 0:m]
    directions = (("shift", np.ones_like(chi)), ("anomaly", chi - chi.mean()),
                  ("x mode", np.cos(2 * np.pi * ii / m + 0.3)), ("y mode", np.cos(np.pi * (jj + 0.5) / n)))
    for name, v in directions:
        h = 1e-7 * np.abs(chi).max() / np.abs(v).max()
        fd = (gpu_loss(P, theta, chi + h * v, target, 100) - gpu_loss(P, theta, chi - h * v, target, 100)) / (2 * h)
        ad = float(np.sum(gc * v))
        assert rel(ad, fd) < TOL, (name, ad, fd)


def test_gradients_vs_oracle_fd():
    """FP64 CPU gradient: five-point central differences of the oracle's loss."""
    from oracle.bind import OracleSim
    N, steps = 32, 100
    P, chi, theta, target = make_case(N, steps, seed=3)
    _, gp, _ = gpu_grad(P, theta, chi, target, steps)
    w = ((P.bx - P.ax) / P.m) * ((P.by - P.ay) / P.n)

    def oracle_loss(th):
        o = OracleSim(with_params(P, th), chi)
        o.set_tolerance(_lib.TOL_RELATIVE, 1e-13)
        o.steps(ADJOINT_DT, steps)
        e = o.eps_pl.reshape(P.n, P.m)
        o.close()
        return w * float(np.sum((e - target) ** 2))

    for k, name in enumerate(PARAM_NAMES):
        h = 1e-4 * abs(theta[k])
        f = []
        for c in (-2, -1, 1, 2):
            t = theta.copy()
            t[k] += c * h
            f.append(oracle_loss(t))
        fd = (f[0] - 8 * f[1] + 8 * f[2] - f[3]) / (12 * h)
        assert rel(gp[k], fd) < TOL, (name, gp[k], fd)


def test_checkpoint_interval_and_scaling(case64):
    P, chi, theta, target = case64
    L1, g1, c1 = gpu_grad(P, theta, chi, target, 100, every=10)
    L2, g2, c2 = gpu_grad(P, theta, chi, target, 100, every=7)
    L3, g3, c3 = gpu_grad(P, theta, chi, target, 100, every=100, dloss=2.5)
    assert rel(L1, L2) < 1e-12 and rel(L1, L3) < 1e-12
    np.testing.assert_allclose(g2, g1, rtol=1e-10)
    np.testing.assert_allclose(g3, 2.5 * g1, rtol=1e-10)
    scale = np.abs(c1).max()
    assert np.abs(c2 - c1).max() < 1e-10 * scale
    assert np.abs(c3 - 2.5 * c1).max() < 1e-10 * scale


def test_backward_twice_and_state_left_at_end(case64):
    """Segments recomputed from checkpoints repeat the forward run exactly, so
    two backward calls agree up to the summation order of atomic adds."""
    P, chi, theta, target = case64
    with ShearSim(with_params(P, theta), chi, **SOLVER) as sim:
        adj = StepAdjoint(sim, ADJOINT_DT, 100, 10)
        adj.forward(target)
        end = sim.get("eps_pl")
        t_end = sim.time
        g1, c1 = adj.backward()
        g2, c2 = adj.backward()
        np.testing.assert_allclose(g2, g1, rtol=1e-12)
        assert np.abs(c2 - c1).max() <= 1e-12 * np.abs(c1).max()
        np.testing.assert_array_equal(sim.get("eps_pl"), end)
        assert sim.time == t_end
        # the handle keeps stepping from the forward run's end state
        sim.steps(ADJOINT_DT, 1)
        assert sim.time > t_end


def test_mixed_precision_forward(case64):
    """The adjoint also runs on a mixed-precision handle (FP64 adjoint solve)."""
    P, chi, theta, target = case64
    _, g64, c64 = gpu_grad(P, theta, chi, target, 100)
    _, g32, c32 = gpu_grad(P, theta, chi, target, 100, precision=_lib.MIXED)
    np.testing.assert_allclose(g32, g64, rtol=1e-7)
    assert np.abs(c32 - c64).max() < 1e-7 * np.abs(c64).max()


def test_autograd_function(case64):
    import torch
    P, chi, theta, target = case64
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    c0 = torch.tensor(chi, dtype=torch.float64, requires_grad=True)
    loss = PlasticStrainLoss.apply(th, c0, P, target, ADJOINT_DT, 100, 10, SOLVER)
    (3.0 * loss).backward()
    L, gp, gc = gpu_grad(P, theta, chi, target, 100)
    assert rel(loss.item(), L) < 1e-12
    np.testing.assert_allclose(th.grad.numpy(), 3.0 * gp, rtol=1e-10)
    assert np.abs(c0.grad.numpy() - 3.0 * gc).max() < 1e-10 * np.abs(gc).max()


def test_adjoint_errors(case64):
    P, chi, theta, target = case64
    with ShearSim(P, chi) as sim:
        with pytest.raises(_lib.StzgError) as e:
            StepAdjoint(sim, ADJOINT_DT, 10).backward()
        assert e.value.status == EINVAL
    with ShearSim(P.copy(chi_diff=0.01), chi) as sim:
        with pytest.raises(_lib.StzgError) as e:
            StepAdjoint(sim, ADJOINT_DT, 10).forward(target)
        assert e.value.status == EINVAL
    with ShearSim(P, chi, track_plastic=False) as sim:
        with pytest.raises(_lib.StzgError) as e:
            StepAdjoint(sim, ADJOINT_DT, 10).forward(target)
        assert e.value.status == EINVAL


def test_adjoint_256_config():
    """The 256x256, 100-step, checkpoint-10 case: parameter gradients against
    central differences (step 1e-6) of the GPU forward run, chi gradient
    along the lowest x and y modes (step 1e-7)."""
    P, chi, theta, target = make_case(256, 100)
    L, gp, gc = gpu_grad(P, theta, chi, target, 100)
    for k, name in enumerate(PARAM_NAMES):
        h = 1e-6 * abs(theta[k])
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (gpu_loss(P, tp, chi, target, 100) - gpu_loss(P, tm, chi, target, 100)) / (2 * h)
        assert rel(gp[k], fd) < TOL, (name, gp[k], fd)
    n, m = chi.shape
    jj, ii = np.mgrid[0:n, 0:m]
    for name, v in (("x mode", np.cos(2 * np.pi * ii / m + 0.3)), ("y mode", np.cos(np.pi * (jj + 0.5) / n))):
        h = 1e-7 * np.abs(chi).max()
        fd = (gpu_loss(P, theta, chi + h * v, target, 100) - gpu_loss(P, theta, chi - h * v, target, 100)) / (2 * h)
        assert rel(float(np.sum(gc * v)), fd) < TOL, (name, float(np.sum(gc * v)), fd)
