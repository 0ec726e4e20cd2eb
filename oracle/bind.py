"""ctypes access to the CPU oracle and to the reference build: TEST ONLY.

``OracleSim`` wraps oracle/_build/libstzoracle.so (the C restatement in
oracle/stz_oracle.c, built by ``build_oracle``); ``ReferenceSim`` wraps
oracle/_ref/libstzref.so, the reference's own shear_sim compiled from its
sources by oracle/build_ref.sh (only where the reference tree is present).
Both expose the same methods, so tests can run either side by side.
Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU leg.
"""
import ctypes
import os
import subprocess

import numpy as np

from stz_gb300.params import StzParams

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libstzoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libstzref.so")
_root = []


def reference_root():
    """The reference tree oracle/build_ref.sh resolves (STZ_REFERENCE_ROOT or
    the recipe's default), or None where it is absent (the GPU host)."""
    if not _root:
        r = subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), "--root"], capture_output=True, text=True)
        _root.append(r.stdout.strip() if r.returncode == 0 and r.stdout.strip() else None)
    return _root[0]

FIELD_IDS = {"u": 0, "v": 1, "p": 2, "q": 3, "s": 4, "tau": 5, "chi": 6, "X": 7, "Y": 8, "ddev": 9}
NODE_FIELDS = ("u", "v", "X", "Y")

_P = ctypes.POINTER(ctypes.c_double)
_libs = {}


def build_oracle(force=False):
    """Compile oracle/stz_oracle.c (plain C, OpenMP) into oracle/_build."""
    if os.path.exists(ORACLE_SO) and not force:
        src = os.path.join(HERE, "stz_oracle.c")
        if os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src):
            return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
           "-o", ORACLE_SO, os.path.join(HERE, "stz_oracle.c"), "-lm"]
    subprocess.check_call(cmd)
    return ORACLE_SO


def build_reference(force=False):
    """Build oracle/_ref/libstzref.so from the reference sources if present."""
    if os.path.exists(REF_SO) and not force:
        return REF_SO
    root = reference_root()
    if root is None:
        return None
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), root])
    return REF_SO


def reference_available():
    return os.path.exists(REF_SO) or reference_root() is not None


def _load(path, prefix):
    if path in _libs:
        return _libs[path]
    lib = ctypes.CDLL(path)
    f = lambda name: getattr(lib, prefix + name)  # noqa: E731
    f("create").restype = ctypes.c_void_p
    f("create").argtypes = [ctypes.POINTER(StzParams)]
    f("destroy").argtypes = [ctypes.c_void_p]
    f("set_state").argtypes = [ctypes.c_void_p, _P]
    f("steps").restype = ctypes.c_long
    f("steps").argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, _P, _P]
    f("steps_direct").argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, _P]
    f("advance_direct").restype = ctypes.c_long
    f("advance_direct").argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _P]
    f("time").restype = ctypes.c_double
    f("time").argtypes = [ctypes.c_void_p]
    f("get").argtypes = [ctypes.c_void_p, ctypes.c_int, _P]
    f("get_vel").argtypes = [ctypes.c_void_p, _P]
    f("mg_levels").restype = ctypes.c_int
    f("mg_levels").argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
    f("mg_stencil").argtypes = [ctypes.c_void_p, ctypes.c_int, _P]
    f("mg_solve").restype = ctypes.c_int
    f("mg_solve").argtypes = [ctypes.c_void_p, ctypes.c_double, _P, _P, ctypes.POINTER(ctypes.c_int)]
    f("mg_vcycle").argtypes = [ctypes.c_void_p, ctypes.c_double, _P, _P]
    f("mg_l2_error").restype = ctypes.c_double
    f("mg_l2_error").argtypes = [ctypes.c_void_p]
    f("init_fields").argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
    f("chi_bicubic").argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _P, ctypes.c_double, ctypes.c_double]
    f("l2_comparison").argtypes = [ctypes.c_void_p, ctypes.c_void_p, _P]
    if prefix == "stzo_":
        lib.stzo_set_tolerance.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        lib.stzo_random_chi.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong, _P]
        lib.stzo_threads.restype = ctypes.c_int
        lib.stzo_set.argtypes = [ctypes.c_void_p, ctypes.c_int, _P]
        lib.stzo_set_threads.argtypes = [ctypes.c_int]
        lib.stzo_mg_residual_sqnorms.argtypes = [ctypes.c_void_p, ctypes.c_double, _P, _P, _P]
    else:
        lib.stzref_output.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
        lib.stzref_qs_measure.argtypes = [ctypes.c_void_p, ctypes.c_int, _P, _P]
        lib.stzref_tractions.argtypes = [ctypes.c_void_p, _P]
        lib.stzref_compute_strain.argtypes = [ctypes.c_void_p, _P]
        lib.stzref_clear_cu.argtypes = [ctypes.c_void_p]
        lib.stzref_set_acc_mult.argtypes = [ctypes.c_void_p, ctypes.c_double]
        lib.stzref_get_acc.restype = ctypes.c_double
        lib.stzref_get_acc.argtypes = [ctypes.c_void_p]
    _libs[path] = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(_P)


class _Sim:
    prefix = None

    def __init__(self, params: StzParams, chi=None):
        self.params = params.copy()
        self.m, self.n = params.m, params.n
        self._f = lambda name: getattr(self.lib, self.prefix + name)  # noqa: E731
        self.h = self._f("create")(ctypes.byref(self.params))
        self.eps_pl = np.zeros(self.m * self.n)
        self.cycles = 0
        self.seconds = 0.0
        if chi is not None:
            self.set_state(chi)

    def close(self):
        if self.h:
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, chi):
        chi = np.ascontiguousarray(chi, dtype=np.float64).reshape(self.n, self.m)
        self._f("set_state")(self.h, _ptr(chi))
        self.eps_pl[:] = 0

    def init_fields(self, chi_case, tem_base=600.0, tem_delta=200.0):
        """shear_sim::init_fields (shear_sim.cc:60-114)."""
        self._f("init_fields")(self.h, int(chi_case), float(tem_base), float(tem_delta))
        self.eps_pl[:] = 0

    def chi_bicubic(self, arr, lo=0.0, sca=1.0):
        """shear_sim::initialize_chi_bicubic (shear_sim.cc:832-909); arr is (nn, mm)."""
        a = np.ascontiguousarray(arr, dtype=np.float64)
        nn, mm = a.shape
        self._f("chi_bicubic")(self.h, mm, nn, _ptr(a), float(lo), float(sca))
        self.eps_pl[:] = 0

    def l2_comparison(self, other):
        """shear_sim::l2_comparison (shear_sim.cc:460-502): (velocity, stress, chi, reference map)."""
        out = np.zeros(4)
        self._f("l2_comparison")(self.h, other.h, _ptr(out))
        return out

    def steps(self, dt, nsteps):
        sec = ctypes.c_double(0)
        c = self._f("steps")(self.h, dt, nsteps, _ptr(self.eps_pl), ctypes.byref(sec))
        if c < 0:
            raise RuntimeError("multigrid solve did not converge")
        self.cycles += c
        self.seconds += sec.value
        return c

    def steps_direct(self, dt, nsteps):
        """Explicit steps (shear_sim::step_forward)."""
        self._f("steps_direct")(self.h, dt, nsteps, _ptr(self.eps_pl))

    def advance_direct(self, dt, target):
        """Explicit steps of dt up to target time (the frame loop of shear_sim::solve)."""
        return self._f("advance_direct")(self.h, dt, target, _ptr(self.eps_pl))

    @property
    def time(self):
        return self._f("time")(self.h)

    def get(self, name):
        """Node fields: (n+1, m); cell fields: (n+2, m) with ghost rows."""
        rows = self.n + 1 if name in NODE_FIELDS else self.n + 2
        out = np.empty(rows * self.m)
        self._f("get")(self.h, FIELD_IDS[name], _ptr(out))
        return out.reshape(rows, self.m)

    def set(self, name, values):
        """Overwrite a stored field (not u, v) in the layout of get()."""
        if name in ("u", "v"):
            raise ValueError("velocities are not settable")
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._f("set")(self.h, FIELD_IDS[name], _ptr(a))

    def fields(self):
        d = {k: self.get(k) for k in FIELD_IDS}
        d["eps_pl"] = self.eps_pl.reshape(self.n, self.m).copy()
        return d

    def vel(self):
        out = np.empty(self.m * (self.n + 1) * 2)
        self._f("get_vel")(self.h, _ptr(out))
        return out.reshape(self.n + 1, self.m, 2)

    def mg_levels(self, dt):
        dims = (ctypes.c_int * 64)()
        nl = self._f("mg_levels")(self.h, dt, dims)
        return [(dims[2 * i], dims[2 * i + 1]) for i in range(nl)]

    def mg_stencil(self, dt, level):
        lv = self.mg_levels(dt)
        mm, nn = lv[level]
        out = np.empty(mm * nn * 10 * 4)
        self._f("mg_stencil")(self.h, level, _ptr(out))
        return out.reshape(nn, mm, 10, 2, 2)

    def mg_solve(self, dt, src, vel):
        src = np.ascontiguousarray(src, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64).copy()
        nc = ctypes.c_int(0)
        ok = self._f("mg_solve")(self.h, dt, _ptr(src), _ptr(vel), ctypes.byref(nc))
        return vel, nc.value, bool(ok)

    def mg_vcycle(self, dt, src, vel):
        src = np.ascontiguousarray(src, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64).copy()
        self._f("mg_vcycle")(self.h, dt, _ptr(src), _ptr(vel))
        return vel

    def mg_l2_error(self):
        return self._f("mg_l2_error")(self.h)


class OracleSim(_Sim):
    prefix = "stzo_"

    def __init__(self, params, chi=None):
        self.lib = _load(build_oracle(), "stzo_")
        super().__init__(params, chi)

    def mg_residual_sqnorms(self, dt, src, vel):
        """(sum of squared residuals, sum of squared sources) of the
        quasi-static system for src and vel, each (n+1, m, 2)."""
        src = np.ascontiguousarray(src, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        out = np.zeros(2)
        self.lib.stzo_mg_residual_sqnorms(self.h, dt, _ptr(src), _ptr(vel), _ptr(out))
        return float(out[0]), float(out[1])

    def set_tolerance(self, mode, value):
        """mode 0: reference rule with multiplier ``value`` (default 1e4);
        mode 1: ||r|| <= value * ||b||."""
        self.lib.stzo_set_tolerance(self.h, mode, value)


class ReferenceSim(_Sim):
    prefix = "stzref_"

    def __init__(self, params, chi=None):
        path = build_reference()
        if path is None:
            raise RuntimeError("reference sources are not available")
        if params.s_y != 1.0:
            raise ValueError("the reference hard-wires the yield stress to 1")
        self.lib = _load(path, "stzref_")
        super().__init__(params, chi)

    def output(self, mode, tmpdir):
        """shear_sim::output of one mode, read back as the float32 matrix."""
        self.lib.stzref_output(self.h, str(tmpdir).encode(), b"f", int(mode), 0)
        path = os.path.join(str(tmpdir), "f.0")
        a = np.fromfile(path, dtype=np.float32)
        os.remove(path)
        w = int(a[0]) + 1
        return a.reshape(-1, w)

    def qs_measure(self, staggered=False):
        q, mx = ctypes.c_double(), ctypes.c_double()
        self.lib.stzref_qs_measure(self.h, int(staggered), ctypes.byref(q), ctypes.byref(mx))
        return q.value, mx.value

    def tractions(self):
        out = np.zeros(4)
        self.lib.stzref_tractions(self.h, _ptr(out))
        return out

    def compute_strain(self):
        out = np.zeros(self.m * self.n)
        self.lib.stzref_compute_strain(self.h, _ptr(out))
        return out.reshape(self.n, self.m)

    def clear_cu(self):
        self.lib.stzref_clear_cu(self.h)

    def set_acc_mult(self, mult):
        self.lib.stzref_set_acc_mult(self.h, mult)

    def set_tolerance(self, mode, value):
        if mode != 0:
            raise ValueError("the reference only has the absolute rule")
        self.set_acc_mult(value)


def random_chi(m, n, l, tem_avg, tem_std, TZ, seed):
    """Seeded chi field from the oracle's restatement of initialize_random."""
    lib = _load(build_oracle(), "stzo_")
    out = np.empty(m * n)
    lib.stzo_random_chi(m, n, l, tem_avg, tem_std, TZ, seed, _ptr(out))
    return out.reshape(n, m)


def oracle_threads():
    lib = _load(build_oracle(), "stzo_")
    return lib.stzo_threads()


def set_oracle_threads(k):
    """OpenMP threads of the oracle's following parallel regions."""
    lib = _load(build_oracle(), "stzo_")
    lib.stzo_set_threads(int(k))
