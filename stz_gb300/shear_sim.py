"""Host-side mirror of the reference's shear_sim / tgmg interfaces over the C ABI.

``ShearSim`` follows esim/sb/main/shear_sim.hh:20-151 (constructor
arguments, step_forward_quasistatic, advection_step, projection_step,
solve_quasistatic, initialize_random, l2_comparison, avg_iters, time) and
``Tgmg`` the multigrid entry points the reference's qs_multi calls
(tgmg.hh:331-351, 439-441).  Both drive the CUDA path in libstzg.so; there is
no CPU path here.
"""
import ctypes

import numpy as np

from . import _lib
from .params import StzParams

FIELD_IDS = {"u": 0, "v": 1, "p": 2, "q": 3, "s": 4, "tau": 5, "chi": 6, "X": 7, "Y": 8, "ddev": 9,
             "eps_pl": 10}
NODE_FIELDS = ("u", "v", "X", "Y")
_P = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_P)


def random_chi(m, n, l, tem_avg, tem_std, TZ, seed):
    """initialize_random semantics (shear_sim.cc:932-984), counter-based seed."""
    out = np.empty(m * n)
    _lib.check(_lib.load().stzg_random_chi(m, n, l, tem_avg, tem_std, TZ, seed, _ptr(out)))
    return out.reshape(n, m)


C_FIELD_DOUBLES = 19  # fields.hh:7-114: u, v, p, q, s, tau, chi, X, Y, ddev, then the update scratch


def c_field_pack(fm_rows, m, n, soa):
    """stzg_c_field_pack: the reference's c_field array (m*(n+2) records of 19
    doubles, rows -1..n) into the up/down buffers p, q, s, tau, chi, X, Y, vel
    (None entries skipped)."""
    rec = np.ascontiguousarray(fm_rows, dtype=np.float64)
    arr = (ctypes.POINTER(ctypes.c_double) * 8)(*[None if a is None else _ptr(a) for a in soa[:8]])
    _lib.check(_lib.load().stzg_c_field_pack(rec.ctypes.data_as(ctypes.c_void_p), m, n, arr))


def c_field_unpack(soa, m, n, fm_rows):
    """stzg_c_field_unpack: the buffers back into the c_field array in place."""
    assert fm_rows.dtype == np.float64 and fm_rows.flags["C_CONTIGUOUS"]
    arr = (ctypes.POINTER(ctypes.c_double) * 8)(*[None if a is None else _ptr(a) for a in soa[:8]])
    _lib.check(_lib.load().stzg_c_field_unpack(arr, m, n, fm_rows.ctypes.data_as(ctypes.c_void_p)))


class ShearSim:
    """One quasi-static STZ simulation on one GPU."""

    def __init__(self, params: StzParams, chi=None, *, precision=_lib.FP64, tol_mode=_lib.TOL_REFERENCE,
                 tol=1e4, track_plastic=True, device=0, inner_cycles=0, use_graphs=True,
                 extrapolate=False, substep_cap=0, advection=_lib.ADV_AUTO):
        lib = _lib.load()
        self.params = params.copy()
        self.m, self.n = params.m, params.n
        self.options = _lib.default_options(precision=precision, tol_mode=tol_mode, tol=tol,
                                            track_plastic=int(track_plastic), device=device,
                                            inner_cycles=inner_cycles, use_graphs=int(use_graphs),
                                            extrapolate=int(extrapolate), substep_cap=int(substep_cap),
                                            advection=int(advection))
        h = ctypes.c_void_p()
        _lib.check(lib.stzg_create(ctypes.byref(self.params), ctypes.byref(self.options), ctypes.byref(h)))
        self.h = h
        self.lib = lib
        self.cycles = 0
        self.stats = _lib.StzgStats()
        if chi is not None:
            self.set_state(chi)

    @classmethod
    def view(cls, handle, params):
        """Non-owning wrapper of a handle that belongs to a batch."""
        self = cls.__new__(cls)
        self.lib = _lib.load()
        self.params = params.copy()
        self.m, self.n = params.m, params.n
        self.h = handle
        self.cycles = 0
        self.stats = _lib.StzgStats()
        self._owned = False
        return self

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None) and getattr(self, "_owned", True):
            self.lib.stzg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state ------------------------------------------------------------
    def set_state(self, chi):
        chi = np.ascontiguousarray(chi, dtype=np.float64).reshape(self.n, self.m)
        _lib.check(self.lib.stzg_set_state(self.h, _ptr(chi)))

    def initialize_random(self, l, tem_avg, tem_stdev, seed=1):
        """shear_sim::initialize_random (shear_sim.cc:932), seeded."""
        chi = random_chi(self.m, self.n, l, tem_avg, tem_stdev, self.params.TZ, seed)
        self.set_state(chi)
        return chi

    def init_fields(self, chi_case, tem_base=600.0, tem_delta=200.0):
        """shear_sim::init_fields (shear_sim.cc:60-114)."""
        _lib.check(self.lib.stzg_init_fields(self.h, int(chi_case), float(tem_base), float(tem_delta)))

    def initialize_chi_bicubic(self, arr, lo=0.0, sca=1.0):
        """shear_sim::initialize_chi_bicubic (shear_sim.cc:832-909); arr is (nn, mm)."""
        a = np.ascontiguousarray(arr, dtype=np.float64)
        nn, mm = a.shape
        _lib.check(self.lib.stzg_chi_bicubic(self.h, mm, nn, _ptr(a), float(lo), float(sca)))

    @property
    def time(self):
        t = ctypes.c_double()
        _lib.check(self.lib.stzg_get_time(self.h, ctypes.byref(t)))
        return t.value

    @time.setter
    def time(self, value):
        _lib.check(self.lib.stzg_set_time(self.h, float(value)))

    def get(self, name):
        """Node fields (n+1, m); cell fields (n+2, m) with ghost rows; eps_pl (n, m)."""
        if name == "eps_pl":
            rows = self.n
        else:
            rows = self.n + 1 if name in NODE_FIELDS else self.n + 2
        out = np.empty(rows * self.m)
        _lib.check(self.lib.stzg_get_field(self.h, FIELD_IDS[name], _ptr(out)))
        return out.reshape(rows, self.m)

    def set(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        _lib.check(self.lib.stzg_set_field(self.h, FIELD_IDS[name], _ptr(a)))

    def fields(self):
        return {k: self.get(k) for k in FIELD_IDS}

    def upload(self, ptrs):
        """Bulk host->device copy of p,q,s,tau,chi,X,Y,vel (raw host addresses)."""
        arr = (ctypes.c_void_p * 8)(*[p or None for p in ptrs[:8]])
        _lib.check(self.lib.stzg_upload(self.h, arr))

    def download(self, ptrs):
        """Bulk device->host copy of p,q,s,tau,chi,X,Y,vel,eps_pl."""
        arr = (ctypes.c_void_p * 9)(*[p or None for p in ptrs[:9]])
        _lib.check(self.lib.stzg_download(self.h, arr))

    def step_host(self, dt, up_ptrs, down_ptrs):
        """One quasi-static step on host-owned fields (stzg_step_qs_host):
        upload p,q,s,tau,chi,X,Y,vel, step, download them and eps_pl."""
        up = (ctypes.c_void_p * 8)(*[p or None for p in up_ptrs[:8]])
        down = (ctypes.c_void_p * 9)(*[p or None for p in down_ptrs[:9]])
        st = _lib.StzgStats()
        _lib.check(self.lib.stzg_step_qs_host(self.h, float(dt), up, down, ctypes.byref(st)))
        self.stats = st
        self.cycles += st.vcycles
        return st.vcycles

    @property
    def mg_persistent(self):
        """Whether the FP32 V-cycle runs its coarse levels and tail in one
        persistent kernel (stzg_get_mg_persistent)."""
        on = ctypes.c_int()
        _lib.check(self.lib.stzg_get_mg_persistent(self.h, ctypes.byref(on)))
        return bool(on.value)

    @mg_persistent.setter
    def mg_persistent(self, on):
        _lib.check(self.lib.stzg_set_mg_persistent(self.h, int(bool(on))))

    def time_kernel(self, dt, kernel, reps=10):
        """Average ms per launch of one kernel group (stzg_time_kernel)."""
        ms = ctypes.c_double()
        _lib.check(self.lib.stzg_time_kernel(self.h, float(dt), int(kernel), int(reps), ctypes.byref(ms)))
        return ms.value

    # -- time stepping ----------------------------------------------------
    def step_forward_quasistatic(self, dt):
        """shear_sim::step_forward_quasistatic (shear_sim.cc:280-291)."""
        return self.steps(dt, 1)

    def steps(self, dt, nsteps):
        st = _lib.StzgStats()
        _lib.check(self.lib.stzg_step_qs(self.h, float(dt), int(nsteps), ctypes.byref(st)))
        self.stats = st
        self.cycles += st.vcycles
        return st.vcycles

    def step_forward(self, dt, nsteps=1):
        """shear_sim::step_forward (shear_sim.cc:185-276): explicit steps."""
        st = _lib.StzgStats()
        _lib.check(self.lib.stzg_step_direct(self.h, float(dt), int(nsteps), ctypes.byref(st)))
        self.stats = st

    def advance_direct(self, dt, target):
        """Explicit steps of dt up to target time (the frame loop of
        shear_sim::solve, shear_sim.cc:120-140); returns the step count."""
        k = ctypes.c_long()
        _lib.check(self.lib.stzg_advance_direct(self.h, float(dt), float(target), ctypes.byref(k)))
        return k.value

    def solve(self, duration, frames, tmult=0.5, frame_callback=None):
        """shear_sim::solve (shear_sim.cc:120-140) without the file output:
        explicit steps of dt = dx^2 * tmult, landing exactly on each frame
        time; frame_callback(k, sim) is called after each frame."""
        dx = (self.params.bx - self.params.ax) / self.m
        dt = dx * dx * tmult
        t_start = self.time
        for k in range(1, frames + 1):
            self.advance_direct(dt, t_start + duration / frames * k)
            if frame_callback:
                frame_callback(k, self)

    # -- frame export and diagnostics --------------------------------------
    def output(self, mode):
        """shear_sim::output (shear_sim.cc:684-720): the Gnuplot binary
        matrix of one field as a float32 array (rows x width)."""
        n = ctypes.c_long()
        _lib.check(self.lib.stzg_output_field(self.h, int(mode), None, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.float32)
        _lib.check(self.lib.stzg_output_field(self.h, int(mode), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                              ctypes.byref(n)))
        return out.reshape(-1, int(out[0]) + 1)

    def write_files(self, directory, frame, flags=4 | 128 | 256 | 512 | 1024):
        """shear_sim::write_files (shear_sim.cc:659-676) into directory."""
        qs = np.zeros(2)
        _lib.check(self.lib.stzg_write_frame(self.h, str(directory).encode(), int(frame), int(flags), _ptr(qs)))
        return qs

    def qs_measure(self, staggered=False):
        """shear_sim::qs_measure (shear_sim.cc:733-775): (Q, max integrand)."""
        q, mx = ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.stzg_qs_measure(self.h, int(staggered), ctypes.byref(q), ctypes.byref(mx)))
        return q.value, mx.value

    def tractions(self):
        """shear_sim::tractions (shear_sim.cc:1003-1028): bottom x, y, top x, y."""
        out = np.zeros(4)
        _lib.check(self.lib.stzg_tractions(self.h, _ptr(out)))
        return out

    def compute_strain(self):
        """shear_sim::compute_strain (shear_sim.cc:778-824): (n, m)."""
        out = np.zeros(self.m * self.n)
        _lib.check(self.lib.stzg_compute_strain(self.h, _ptr(out)))
        return out.reshape(self.n, self.m)

    def advection_step(self, dt):
        _lib.check(self.lib.stzg_advection_step(self.h, float(dt)))

    def projection_step(self, dt):
        st = _lib.StzgStats()
        _lib.check(self.lib.stzg_projection_step(self.h, float(dt), ctypes.byref(st)))

    def solve_quasistatic(self, duration, frames, steps, frame_callback=None):
        """shear_sim::solve_quasistatic (shear_sim.cc:159-181) without the file
        output; frame_callback(k, sim) is called after each frame."""
        dt = duration / frames / steps
        for k in range(1, frames + 1):
            self.steps(dt, steps)
            if frame_callback:
                frame_callback(k, self)

    def avg_iters(self):
        a = ctypes.c_double()
        _lib.check(self.lib.stzg_avg_iters(self.h, ctypes.byref(a)))
        return a.value

    def l2_comparison(self, other):
        """shear_sim::l2_comparison (shear_sim.cc:460-502)."""
        out = np.zeros(4)
        _lib.check(self.lib.stzg_l2_comparison(self.h, other.h, _ptr(out)))
        return out

    # -- multigrid (tgmg drop-in) -----------------------------------------
    def mg_levels(self, dt):
        nl = ctypes.c_int()
        dims = (ctypes.c_int * 32)()
        _lib.check(self.lib.stzg_mg_levels(self.h, float(dt), ctypes.byref(nl), dims))
        return [(dims[2 * i], dims[2 * i + 1]) for i in range(nl.value)]

    def mg_stencil(self, dt, level):
        mm, nn = self.mg_levels(dt)[level]
        out = np.empty(mm * nn * 40)
        _lib.check(self.lib.stzg_mg_stencil(self.h, float(dt), int(level), _ptr(out)))
        return out.reshape(nn, mm, 10, 2, 2)

    def mg_solve(self, dt, src, vel):
        src = np.ascontiguousarray(src, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64).copy()
        nc = ctypes.c_int()
        _lib.check(self.lib.stzg_mg_solve(self.h, float(dt), _ptr(src), _ptr(vel), ctypes.byref(nc)))
        return vel, nc.value, True

    def mg_vcycle(self, dt, src, vel):
        src = np.ascontiguousarray(src, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64).copy()
        _lib.check(self.lib.stzg_mg_vcycle(self.h, float(dt), _ptr(src), _ptr(vel)))
        return vel

    def mg_l2_error(self, dt, src, vel):
        src = np.ascontiguousarray(src, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        e = ctypes.c_double()
        _lib.check(self.lib.stzg_mg_l2_error(self.h, float(dt), _ptr(src), _ptr(vel), ctypes.byref(e)))
        return e.value


class Tgmg:
    """tgmg<qs_multi,vec,mat> drop-in over a ShearSim's operator
    (tgmg.hh:286-495): setup() for a time step, solve_v_cycle() with the
    adaptive predictor, v_cycle(), l2_error()."""

    def __init__(self, sim: ShearSim, dt):
        self.sim = sim
        self.dt = dt

    def setup(self):
        return self.sim.mg_levels(self.dt)

    def solve_v_cycle(self, src, vel):
        return self.sim.mg_solve(self.dt, src, vel)

    def v_cycle(self, src, vel):
        return self.sim.mg_vcycle(self.dt, src, vel)

    def l2_error(self, src, vel):
        return self.sim.mg_l2_error(self.dt, src, vel)
