"""Host-side mirror of the reference's coord_transforms simulation
(esim/coord_transforms/simple_shear/shear_sim.{hh,cc}) over the C ABI in
include/stzg_ct.h: the quasi-static STZ step in coordinates that follow a
simple shear of rate lamb, x periodic and y periodic or walled.  The step runs
on the GPU (libstzg.so); there is no CPU path.
"""
import ctypes
import math

import numpy as np

from . import _lib

EXPORTS = ["stzg_ct_create", "stzg_ct_destroy", "stzg_ct_init_fields", "stzg_ct_chi_bicubic",
           "stzg_ct_compute_strain", "stzg_ct_output_field", "stzg_ct_write_frame", "stzg_ct_solve_quasistatic",
           "stzg_ct_solve", "stzg_ct_l2_comparison_transform", "stzg_ct_set_field", "stzg_ct_get_field",
           "stzg_ct_set_time", "stzg_ct_get_time", "stzg_ct_set_precision", "stzg_ct_set_solve_policy", "stzg_ct_step_qs", "stzg_ct_batch_step_qs", "stzg_ct_step_direct", "stzg_ct_tracers_init",
           "stzg_ct_tracers_update", "stzg_ct_tracers_get"]
FIELDS = ("u", "v", "p", "q", "s", "tau", "chi", "X", "Y", "ddev")
BOLTZMANN = 1.3806503e-23

_P = ctypes.POINTER(ctypes.c_double)


class CtParams(ctypes.Structure):
    """stzg_ct_params: shear_sim's constructor arguments (shear_sim.hh:157-161)
    and the STZ law (stz_model.hh)."""
    _fields_ = [(k, ctypes.c_int) for k in ("m", "n", "y_prd", "stz_model", "t_model")] + \
               [(k, ctypes.c_double) for k in ("ax", "bx", "ay", "by", "mu", "K", "viscosity", "chi_len", "t_scale",
                                               "adapt_fac", "u_bdry", "lamb", "TZ", "c0", "tau0", "kappa", "Delta",
                                               "Omegaeps0", "chi_inf", "theta", "rho")]


def transform_shear(m, n, *, y_prd=True, lamb=None, u_bdry=None, sca=2e4, chi_len=0.1, visc=0.02,
                    adapt_fac=1e-4, stz_model=2, x_half=2.0, y_half=1.0):
    """The configuration of the reference's driver
    (esim/coord_transforms/simple_shear/shear_coord_transform.cc:20-89):
    Vitreloy-1 constants (E 101 GPa, nu 0.35, s_y 0.85 GPa), the linear
    athermal law, y periodic with lamb = 1e-3 and still walls, or walled with
    lamb = 0 and u_bdry = 1e-7 * sca."""
    TZ, kB = 21000.0, BOLTZMANN
    s_y, E, nu = 0.85e9, 101e9, 0.35
    p = CtParams()
    p.m, p.n, p.y_prd, p.stz_model, p.t_model = m, n, int(y_prd), stz_model, -1
    p.ax, p.bx, p.ay, p.by = -x_half, x_half, -y_half, y_half
    p.K = E / (3 * (1 - 2 * nu) * s_y)
    p.mu = E / (2 * (1 + nu) * s_y)
    le, rho0 = 1e-2, 6125
    p.t_scale = le / math.sqrt(p.mu * s_y / rho0) * sca
    p.viscosity, p.chi_len, p.adapt_fac = visc, chi_len, adapt_fac
    if y_prd:
        p.u_bdry = 0.0 if u_bdry is None else u_bdry
        p.lamb = 1e-3 if lamb is None else lamb
    else:
        p.u_bdry = 1e-7 * sca if u_bdry is None else u_bdry
        p.lamb = 0.0 if lamb is None else lamb
    p.TZ = TZ
    p.c0, p.tau0, p.kappa = 0.4, 1e-13, 4.2
    p.Delta = 8000 / TZ
    omega, eps0 = 300. * 22 / 17, 0.3
    p.Omegaeps0 = omega * 1e-30 * eps0 * s_y / (TZ * kB)
    p.chi_inf, p.theta, p.rho = 900 / TZ, 400 / TZ, 0.0
    return p


def load():
    lib = _lib.load()
    if getattr(lib, "_ct_declared", False):
        return lib
    V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    decl = {
        "stzg_ct_create": (I, [ctypes.POINTER(CtParams), I, ctypes.POINTER(V)]),
        "stzg_ct_destroy": (I, [V]),
        "stzg_ct_init_fields": (I, [V, I, D, D]),
        "stzg_ct_chi_bicubic": (I, [V, I, I, ctypes.POINTER(ctypes.c_double), D, D]),
        "stzg_ct_compute_strain": (I, [V, ctypes.POINTER(ctypes.c_double)]),
        "stzg_ct_output_field": (I, [V, I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_long)]),
        "stzg_ct_write_frame": (I, [V, ctypes.c_char_p, I, ctypes.c_uint]),
        "stzg_ct_solve_quasistatic": (I, [V, D, I, I, ctypes.c_char_p, ctypes.c_uint, I]),
        "stzg_ct_solve": (I, [V, D, I, ctypes.c_char_p, ctypes.c_uint, I]),
        "stzg_ct_l2_comparison_transform": (I, [V, V, ctypes.POINTER(ctypes.c_double)]),
        "stzg_ct_set_field": (I, [V, I, _P]),
        "stzg_ct_get_field": (I, [V, I, _P]),
        "stzg_ct_set_time": (I, [V, D]),
        "stzg_ct_set_precision": (I, [V, I]),
        "stzg_ct_set_solve_policy": (I, [V, I]),
        "stzg_ct_get_time": (I, [V, _P]),
        "stzg_ct_step_qs": (I, [V, D, I, ctypes.POINTER(ctypes.c_long), _P]),
        "stzg_ct_batch_step_qs": (I, [ctypes.POINTER(V), I, D, I, I, ctypes.POINTER(ctypes.c_long), _P]),
        "stzg_ct_step_direct": (I, [V, D, I, _P]),
        "stzg_ct_tracers_init": (I, [V, I, I]),
        "stzg_ct_tracers_update": (I, [V, ctypes.POINTER(I)]),
        "stzg_ct_tracers_get": (I, [V, _P, I, ctypes.POINTER(I)]),
    }
    for name, (res, args) in decl.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._ct_declared = True
    return lib


class CtSim:
    """shear_sim of the coord_transforms variant on one GPU."""

    def __init__(self, params, device=0):
        self.lib = load()
        self.P = params
        h = ctypes.c_void_p()
        _lib.check(self.lib.stzg_ct_create(ctypes.byref(params), device, ctypes.byref(h)))
        self.h = h
        self.vcycles = 0
        self.seconds = 0.0

    def close(self):
        if getattr(self, "h", None):
            self.lib.stzg_ct_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_fields(self, chi_case=0, tem_base=600, tem_delta=200):
        _lib.check(self.lib.stzg_ct_init_fields(self.h, chi_case, tem_base, tem_delta))

    def initialize_chi_bicubic(self, arr, lo=0.0, sca=1.0):
        """shear_sim::initialize_chi_bicubic (shear_sim.cc:1067-1134); arr is (nn, mm)."""
        a = np.ascontiguousarray(arr, dtype=np.float64)
        nn, mm = a.shape
        _lib.check(self.lib.stzg_ct_chi_bicubic(self.h, mm, nn, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                float(lo), float(sca)))

    def l2_comparison_transform(self, phys):
        """shear_sim::l2_comparison_transform against a physical-frame run."""
        out = np.zeros(4)
        _lib.check(self.lib.stzg_ct_l2_comparison_transform(self.h, phys.h,
                                                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def compute_strain(self):
        """shear_sim::compute_strain: (6, n+1, m) = E_xx, E_xy, E_yy, trace, second invariant, deviatoric norm."""
        out = np.empty(6 * (self.P.n + 1) * self.P.m)
        _lib.check(self.lib.stzg_ct_compute_strain(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out.reshape(6, self.P.n + 1, self.P.m)

    def output(self, mode):
        """shear_sim::output of one mode as the float32 matrix the reference writes."""
        n = ctypes.c_long()
        _lib.check(self.lib.stzg_ct_output_field(self.h, int(mode), None, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.float32)
        _lib.check(self.lib.stzg_ct_output_field(self.h, int(mode), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                 ctypes.byref(n)))
        return out.reshape(-1, int(out[0]) + 1)

    def write_files(self, directory, frame, fflags):
        """shear_sim::write_files into `directory` with the reference's flags."""
        _lib.check(self.lib.stzg_ct_write_frame(self.h, str(directory).encode(), int(frame), int(fflags)))

    def solve_quasistatic(self, duration, frames, steps, directory, fflags, verbose=False):
        _lib.check(self.lib.stzg_ct_solve_quasistatic(self.h, float(duration), int(frames), int(steps),
                                                      str(directory).encode(), int(fflags), int(verbose)))

    def solve(self, duration, frames, directory, fflags, verbose=False):
        _lib.check(self.lib.stzg_ct_solve(self.h, float(duration), int(frames), str(directory).encode(),
                                          int(fflags), int(verbose)))

    def get(self, name):
        out = np.empty((self.P.n + 1, self.P.m))
        _lib.check(self.lib.stzg_ct_get_field(self.h, FIELDS.index(name), out.ctypes.data_as(_P)))
        return out

    def set(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _lib.check(self.lib.stzg_ct_set_field(self.h, FIELDS.index(name), a.ctypes.data_as(_P)))

    def fields(self):
        return {k: self.get(k) for k in FIELDS}

    @property
    def time(self):
        t = ctypes.c_double()
        _lib.check(self.lib.stzg_ct_get_time(self.h, ctypes.byref(t)))
        return t.value

    @time.setter
    def time(self, t):
        _lib.check(self.lib.stzg_ct_set_time(self.h, float(t)))

    def set_precision(self, mixed):
        """mixed: the projection solves with FP32 V-cycles inside FP64
        refinement, to the same threshold on the FP64 residual."""
        _lib.check(self.lib.stzg_ct_set_precision(self.h, 1 if mixed else 0))

    def set_solve_policy(self, checked):
        """checked: the projection runs V-cycles until its residual meets the
        threshold (tested after each) instead of the predictor's counts."""
        _lib.check(self.lib.stzg_ct_set_solve_policy(self.h, 1 if checked else 0))

    def step_forward_quasistatic(self, dt, nsteps=1):
        vc, sec = ctypes.c_long(), ctypes.c_double()
        _lib.check(self.lib.stzg_ct_step_qs(self.h, float(dt), int(nsteps), ctypes.byref(vc), ctypes.byref(sec)))
        self.vcycles, self.seconds = vc.value, sec.value

    def step_forward(self, dt, nsteps=1):
        """shear_sim::step_forward (shear_sim.cc:218-349), the explicit step."""
        sec = ctypes.c_double()
        _lib.check(self.lib.stzg_ct_step_direct(self.h, float(dt), int(nsteps), ctypes.byref(sec)))
        self.seconds = sec.value

    # -- Lagrangian tracers (shear_sim.cc:1247-1355) ------------------------
    def initialize_tracers(self, mm, nn):
        """shear_sim::initialize_tracers(mm, nn)."""
        _lib.check(self.lib.stzg_ct_tracers_init(self.h, int(mm), int(nn)))

    def update_tracers(self):
        """shear_sim::update_tracers(); returns the number of tracers dropped."""
        lost = ctypes.c_int()
        _lib.check(self.lib.stzg_ct_tracers_update(self.h, ctypes.byref(lost)))
        return lost.value

    def tracers(self):
        """(count, 6) array: reference point, position, velocity estimate."""
        cnt = ctypes.c_int()
        _lib.check(self.lib.stzg_ct_tracers_get(self.h, None, 0, ctypes.byref(cnt)))
        out = np.empty((cnt.value, 6))
        if cnt.value:
            _lib.check(self.lib.stzg_ct_tracers_get(self.h, out.ctypes.data_as(_P), cnt.value, ctypes.byref(cnt)))
        return out


def batch_step_qs(sims, dt, nsteps, threads=0):
    """stzg_ct_batch_step_qs: advance independent CtSim handles together (one
    host thread per handle up to `threads`, own streams).  Returns (vcycles per
    handle, wall seconds)."""
    lib = load()
    hs = (ctypes.c_void_p * len(sims))(*[s.h.value for s in sims])
    vc = (ctypes.c_long * len(sims))()
    sec = ctypes.c_double()
    _lib.check(lib.stzg_ct_batch_step_qs(hs, len(sims), float(dt), int(nsteps), int(threads), vc, ctypes.byref(sec)))
    for s, v in zip(sims, vc):
        s.vcycles = v
    return list(vc), sec.value
