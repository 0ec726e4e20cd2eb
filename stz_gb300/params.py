"""Simulation parameters of the quasi-static STZ step (C layout of stz_params).

Mirrors the constructor arguments of the reference's ``shear_sim``
(esim/sb/main/shear_sim.hh:95-99) and its STZ law classes
(esim/sb/main/stz_model.hh:9-207), flattened into one plain struct that the
C ABI takes by pointer.  ``s_y`` is the yield stress; the reference hard-wires
it to 1 (stz_model.hh:26 ``s0(1)``, ``if(sbar<1)``).
"""
import ctypes

STZ_LINEAR = 0
STZ_NONLINEAR = 1
STZ_LINEAR_ATHERMAL = 2
STZ_NONLINEAR_ATHERMAL = 3

BOLTZMANN = 1.3806503e-23  # value used by the reference drivers (shear_test.cc:14)


class StzParams(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int), ("n", ctypes.c_int),
        ("stz_model", ctypes.c_int), ("t_model", ctypes.c_int),
        ("ax", ctypes.c_double), ("bx", ctypes.c_double),
        ("ay", ctypes.c_double), ("by", ctypes.c_double),
        ("mu", ctypes.c_double), ("K", ctypes.c_double), ("viscosity", ctypes.c_double),
        ("chi_diff", ctypes.c_double), ("chi_len", ctypes.c_double),
        ("t_scale", ctypes.c_double), ("adapt_fac", ctypes.c_double), ("u_bdry", ctypes.c_double),
        ("TZ", ctypes.c_double), ("c0", ctypes.c_double), ("tau0", ctypes.c_double),
        ("kappa", ctypes.c_double), ("Delta", ctypes.c_double), ("Omegaeps0", ctypes.c_double),
        ("chi_inf", ctypes.c_double), ("theta", ctypes.c_double), ("rho", ctypes.c_double),
        ("s_y", ctypes.c_double),
    ]

    def copy(self, **changes):
        p = StzParams()
        ctypes.pointer(p)[0] = self
        for k, v in changes.items():
            setattr(p, k, v)
        return p

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def simple_shear(N, M=None, *, u_bdry=1e-4, c0=0.4, eps0=1.0, chi_inf_K=900.0, s_y=1.0,
                 stz_model=STZ_LINEAR_ATHERMAL, t_model=-1, t_scale=1.0, viscosity=0.0,
                 chi_diff=0.0, chi_len=0.0, adapt_fac=0.002, mu=1.0, K=2.5, x_half=None):
    """Simple shear on [-x_half,x_half]x[-1,1], periodic in x, walls moving at +-u_bdry.

    x_half defaults to N/M, i.e. square cells (dx == dy): the reference's
    coarse-grid entries (qs_multi.hh:26-29) only match its applied operator
    (qs_multi.hh:41-50) for square cells, and its multigrid diverges otherwise.

    STZ constants follow the reference driver shear_test.cc:30-39 (T_Z=21000,
    tau0=1e-13, kappa=4.2, Delta=8000/T_Z, Omega=300 A^3, theta=400/T_Z) with
    the strain scale eps0 and Omega*eps0 = Omega*1e-30*eps0*1.1e9/(T_Z k_B).
    """
    TZ = 21000.0
    p = StzParams()
    p.m = N
    p.n = N if M is None else M
    p.stz_model = stz_model
    p.t_model = t_model
    xh = (p.m / p.n) if x_half is None else x_half
    p.ax, p.bx, p.ay, p.by = -xh, xh, -1.0, 1.0
    p.mu, p.K, p.viscosity = mu, K, viscosity
    p.chi_diff, p.chi_len = chi_diff, chi_len
    p.t_scale, p.adapt_fac, p.u_bdry = t_scale, adapt_fac, u_bdry
    p.TZ = TZ
    p.c0 = c0
    p.tau0 = 1e-13
    p.kappa = 4.2
    p.Delta = 8000.0 / TZ
    p.Omegaeps0 = 300.0 * 1e-30 * eps0 * 1.1e9 / (TZ * BOLTZMANN)
    p.chi_inf = chi_inf_K / TZ
    p.theta = 400.0 / TZ
    p.rho = 0.0
    p.s_y = s_y
    return p


def plastic_shear(N, M=None, **kw):
    """Plastic-active variant: walls fast enough that the whole layer yields.

    The reference-like configurations stay far below yield (maximum deviatoric
    stress ~1.5e-4 for u_bdry=1e-4), so they never exercise the STZ law.  With
    u_bdry=4 the wall displacement passes the yield strain at t~0.7.
    """
    kw.setdefault("u_bdry", 4.0)
    return simple_shear(N, M, **kw)


def adjoint_shear(N, M=None, **kw):
    """Plastic-active shear for gradient checks: 100 steps of ADJOINT_DT.

    Linear thermal STZ law (stz_model.hh:58-67), which has no yield kink.
    Walls at +-8 with the ramp u = 8 t reach a CFL number of 0.41 at t = 0.2
    on a 256-cell line; the stress scale s_y = 0.1 is passed at t ~ 0.14 and
    t_scale = 3e5 makes the plastic strain reach ~3e-2 in the most active
    cells.  adapt_fac = 0.02 keeps every cell at one plastic sub-step per
    step (the largest stress drop per step is ~1.4e-2), so the loss is smooth
    in c0, Omega*eps0, chi_inf, s_y and chi at the scale of a 1e-6 relative
    finite-difference step.  With the sub-stepping active (adapt_fac 0.002,
    or the athermal law at t_scale 1e9 with hundreds of sub-steps) the step
    count of some cell changes under parameter changes of 1e-7 and the
    discrete map is only piecewise smooth at that scale.  At the reference
    wall speed 1e-4 the layer never yields and every gradient is zero.
    """
    kw.setdefault("u_bdry", 8.0)
    kw.setdefault("s_y", 0.1)
    kw.setdefault("t_scale", 3e5)
    kw.setdefault("stz_model", STZ_LINEAR)
    kw.setdefault("adapt_fac", 0.02)
    return simple_shear(N, M, **kw)


ADJOINT_DT = 2e-3


def default_dt(N):
    """Time step of the reference-like configurations (dt=1e-2)."""
    return 1e-2


def cfl(p, dt):
    """Advective CFL number of the wall speed on the grid."""
    return abs(p.u_bdry) * dt * p.m / (p.bx - p.ax)


__all__ = ["StzParams", "simple_shear", "plastic_shear", "adjoint_shear", "ADJOINT_DT", "default_dt", "cfl",
           "STZ_LINEAR", "STZ_NONLINEAR", "STZ_LINEAR_ATHERMAL", "STZ_NONLINEAR_ATHERMAL"]
