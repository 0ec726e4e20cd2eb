"""ctypes access to the reference's general multigrid build: TEST ONLY.

``ReferenceTgmg`` wraps oracle/_ref/libtgmgref.so, the reference's own
tgmg<poisson_fd,double,double> compiled from its sources by
oracle/build_ref.sh together with oracle/ref_tgmg_driver.cc (only where the
reference tree is present).  Imported only by tests/ and the golden-fixture
script.
"""
import ctypes
import os

import numpy as np

from oracle.bind import build_reference, reference_root

HERE = os.path.dirname(os.path.abspath(__file__))
TGMG_REF_SO = os.path.join(HERE, "_ref", "libtgmgref.so")

_P = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_lib = None


def available():
    if os.path.exists(TGMG_REF_SO):
        return True
    if reference_root() is None:
        return False
    build_reference(force=True)
    return os.path.exists(TGMG_REF_SO)


def _load():
    global _lib
    if _lib is None:
        if not available():
            raise OSError("reference multigrid build unavailable")
        L = ctypes.CDLL(TGMG_REF_SO)
        V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.tgref_create.restype = V
        L.tgref_create.argtypes = [I, I, D, D, D, D]
        L.tgref_destroy.argtypes = [V]
        for f in ("tgref_set_b", "tgref_get_b", "tgref_set_z", "tgref_get_z"):
            getattr(L, f).argtypes = [V, _P]
        L.tgref_gaussian.argtypes = [V, D, D, D, D]
        L.tgref_solve.argtypes = [V, I, _IP, _IP]
        L.tgref_solve_fixed.argtypes = [V]
        L.tgref_vcycles.argtypes = [V, I]
        L.tgref_l2.restype = D
        L.tgref_l2.argtypes = [V]
        L.tgref_acc.restype = D
        L.tgref_acc.argtypes = [V]
        L.tgref_levels.argtypes = [V, _IP]
        L.tgref_stencil.argtypes = [V, I, _P]
        L.tgref_time_rotating.restype = D
        L.tgref_time_rotating.argtypes = [V, I, _IP]
        _lib = L
    return _lib


class ReferenceTgmg:
    """poisson_fd + tgmg<poisson_fd,double,double> + a tgmg_predict."""

    def __init__(self, m, n, ax, bx, ay, by):
        self.L = _load()
        self.m, self.n = m, n
        self.h = self.L.tgref_create(m, n, ax, bx, ay, by)

    def close(self):
        if self.h:
            self.L.tgref_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def acc(self):
        return self.L.tgref_acc(self.h)

    def _get(self, f):
        a = np.empty((self.n, self.m))
        f(self.h, a.ctypes.data_as(_P))
        return a

    def b(self):
        return self._get(self.L.tgref_get_b)

    def z(self):
        return self._get(self.L.tgref_get_z)

    def set_b(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        self.L.tgref_set_b(self.h, b.ctypes.data_as(_P))

    def set_z(self, z):
        z = np.ascontiguousarray(z, dtype=np.float64)
        self.L.tgref_set_z(self.h, z.ctypes.data_as(_P))

    def gaussian_source_term(self, gx, gy, r, amp):
        self.L.tgref_gaussian(self.h, gx, gy, r, amp)

    def solve(self, kind=4):
        it, lim = ctypes.c_int(), ctypes.c_int()
        ok = self.L.tgref_solve(self.h, kind, ctypes.byref(it), ctypes.byref(lim))
        return bool(ok), it.value, lim.value

    def v_cycles(self, count):
        self.L.tgref_vcycles(self.h, count)

    def l2_error(self):
        return self.L.tgref_l2(self.h)

    def levels(self):
        dims = np.zeros(40, dtype=np.int32)
        nl = self.L.tgref_levels(self.h, dims.ctypes.data_as(_IP))
        return [(int(dims[2 * k]), int(dims[2 * k + 1])) for k in range(nl)]

    def stencil(self, level):
        m, n = self.levels()[level]
        out = np.empty((n, m, 10))
        self.L.tgref_stencil(self.h, level, out.ctypes.data_as(_P))
        return out

    def time_rotating(self, trials):
        vc = ctypes.c_int()
        t = self.L.tgref_time_rotating(self.h, trials, ctypes.byref(vc))
        return t, vc.value
