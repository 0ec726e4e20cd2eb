"""Gradients of the quasi-static STZ simulation over the C ABI.

``StepAdjoint`` drives the forward/backward pair stzg_adjoint_forward /
stzg_adjoint_backward on one ShearSim: the forward pass runs ``nsteps``
steps of shear_sim::step_forward_quasistatic (shear_sim.cc:280-291) with a
checkpoint every ``checkpoint_every`` steps and returns

    L = dx dy sum_cells (eps_pl - target)^2,

the backward pass returns dL/d(c0, Omega*eps0, chi_inf, s_y) and dL/d chi at
t = 0 from the hand-written adjoint with checkpointed recomputation.

``PlasticStrainLoss`` wraps the pair as a torch.autograd.Function of the four
parameters and the initial chi field.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .params import StzParams
from .shear_sim import ShearSim

PARAM_NAMES = ("c0", "Omegaeps0", "chi_inf", "s_y")
_P = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_P)


class StepAdjoint:
    """Forward/backward pair on one simulation handle."""

    def __init__(self, sim: ShearSim, dt, nsteps, checkpoint_every=10):
        self.sim = sim
        self.dt = float(dt)
        self.nsteps = int(nsteps)
        self.every = int(checkpoint_every)
        self.loss = None

    def forward(self, target):
        """Steps the simulation and returns the loss against target (n, m)."""
        tgt = np.ascontiguousarray(target, dtype=np.float64).reshape(self.sim.n, self.sim.m)
        loss = ctypes.c_double()
        _lib.check(self.sim.lib.stzg_adjoint_forward(self.sim.h, self.dt, self.nsteps, self.every, _ptr(tgt),
                                                      ctypes.byref(loss)))
        self.loss = loss.value
        return self.loss

    def backward(self, dloss=1.0):
        """Returns (dloss * dL/dparams [4], dloss * dL/dchi0 (n, m))."""
        gp = np.zeros(4)
        gc = np.zeros(self.sim.n * self.sim.m)
        _lib.check(self.sim.lib.stzg_adjoint_backward(self.sim.h, float(dloss), _ptr(gp), _ptr(gc)))
        return gp, gc.reshape(self.sim.n, self.sim.m)


def with_params(params: StzParams, theta):
    """Copy of params with (c0, Omega*eps0, chi_inf, s_y) = theta."""
    return params.copy(**{k: float(v) for k, v in zip(PARAM_NAMES, theta)})


class PlasticStrainLoss(torch.autograd.Function):
    """loss = PlasticStrainLoss.apply(theta, chi0, params, target, dt, nsteps, every, sim_kw)

    theta: float64 tensor (c0, Omega*eps0, chi_inf, s_y); chi0: float64 (n, m)
    initial effective temperature.  Each forward call creates a handle with
    those values, runs the forward pass and keeps the handle for backward.
    """

    @staticmethod
    def forward(ctx, theta, chi0, params, target, dt, nsteps, every=10, sim_kw=None):
        P = with_params(params, theta.detach().cpu().double().numpy())
        sim = ShearSim(P, chi0.detach().cpu().double().numpy(), **(sim_kw or {}))
        adj = StepAdjoint(sim, dt, nsteps, every)
        loss = adj.forward(np.asarray(target))
        ctx.adj = adj
        ctx.devs = (theta.device, chi0.device)
        return torch.tensor(loss, dtype=torch.float64, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        adj = ctx.adj
        gp, gc = adj.backward(float(grad_out))
        adj.sim.close()
        ctx.adj = None
        return (torch.from_numpy(gp).to(ctx.devs[0]), torch.from_numpy(gc).to(ctx.devs[1]),
                None, None, None, None, None, None)
