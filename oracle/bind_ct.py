"""ctypes access to the reference's coord_transforms simulation: TEST ONLY.

``ReferenceCt`` wraps oracle/_ref/libctref.so, the reference's own
esim/coord_transforms/simple_shear shear_sim compiled from its sources by
oracle/build_ref.sh with oracle/ref_ct_driver.cc (only where the reference
tree is present).  Imported only by tests/ and the golden-fixture script.
"""
import ctypes
import os

import numpy as np

from oracle.bind import build_reference, reference_root

HERE = os.path.dirname(os.path.abspath(__file__))
CT_REF_SO = os.path.join(HERE, "_ref", "libctref.so")
FIELDS = ("u", "v", "p", "q", "s", "tau", "chi", "X", "Y", "ddev")

_P = ctypes.POINTER(ctypes.c_double)
_lib = None


def available():
    if os.path.exists(CT_REF_SO):
        return True
    if reference_root() is None:
        return False
    build_reference(force=True)
    return os.path.exists(CT_REF_SO)


def _load():
    global _lib
    if _lib is None:
        if not available():
            raise OSError("reference coord_transforms build unavailable")
        from stz_gb300.ct_sim import CtParams
        L = ctypes.CDLL(CT_REF_SO)
        V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.ctref_create.restype = V
        L.ctref_create.argtypes = [ctypes.POINTER(CtParams)]
        L.ctref_destroy.argtypes = [V]
        L.ctref_init_fields.argtypes = [V, I, D, D]
        L.ctref_chi_bicubic.argtypes = [V, I, I, _P, D, D]
        L.ctref_write_files.argtypes = [V, ctypes.c_char_p, I, ctypes.c_uint]
        L.ctref_l2_comparison_transform.argtypes = [V, V, _P]
        L.ctref_get_field.argtypes = [V, I, _P]
        L.ctref_set_field.argtypes = [V, I, _P]
        L.ctref_steps.argtypes = [V, D, I]
        L.ctref_steps_direct.argtypes = [V, D, I]
        L.ctref_set_time.argtypes = [V, D]
        L.ctref_time.restype = D
        L.ctref_time.argtypes = [V]
        L.ctref_vcount.restype = I
        L.ctref_vcount.argtypes = [V]
        L.ctref_init_tracers.argtypes = [V, I, I]
        L.ctref_update_tracers.argtypes = [V]
        L.ctref_get_tracers.restype = I
        L.ctref_get_tracers.argtypes = [V, _P, I]
        _lib = L
    return _lib


class ReferenceCt:
    def __init__(self, params):
        self.L = _load()
        self.P = params
        self.h = self.L.ctref_create(ctypes.byref(params))

    def close(self):
        if self.h:
            self.L.ctref_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_fields(self, chi_case, base, delta):
        self.L.ctref_init_fields(self.h, chi_case, base, delta)

    def l2_comparison_transform(self, phys):
        out = np.zeros(4)
        self.L.ctref_l2_comparison_transform(self.h, phys.h, out.ctypes.data_as(_P))
        return out

    def write_files(self, directory, k, fflags):
        self.L.ctref_write_files(self.h, str(directory).encode(), k, fflags)

    def chi_bicubic(self, arr, lo, sca):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        nn, mm = a.shape
        self.L.ctref_chi_bicubic(self.h, mm, nn, a.ctypes.data_as(_P), lo, sca)

    def get(self, name):
        out = np.empty((self.P.n + 1, self.P.m))
        self.L.ctref_get_field(self.h, FIELDS.index(name), out.ctypes.data_as(_P))
        return out

    def set(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.L.ctref_set_field(self.h, FIELDS.index(name), a.ctypes.data_as(_P))

    def fields(self):
        return {k: self.get(k) for k in FIELDS}

    def steps(self, dt, k):
        self.L.ctref_steps(self.h, dt, k)

    @property
    def time(self):
        return self.L.ctref_time(self.h)

    @property
    def vcount(self):
        return self.L.ctref_vcount(self.h)

    def initialize_tracers(self, mm, nn):
        self.L.ctref_init_tracers(self.h, mm, nn)

    def update_tracers(self):
        self.L.ctref_update_tracers(self.h)

    def tracers(self):
        n = self.L.ctref_get_tracers(self.h, None, 0)
        out = np.empty((n, 6))
        if n:
            self.L.ctref_get_tracers(self.h, out.ctypes.data_as(_P), n)
        return out

    def step_forward(self, dt, k=1):
        self.L.ctref_steps_direct(self.h, dt, k)

    def set_time(self, t):
        self.L.ctref_set_time(self.h, t)
