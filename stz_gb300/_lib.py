"""ctypes binding of the C ABI in include/stzg.h (libstzg.so).

The library is loaded from stz_gb300/_build/libstzg.so (built in-tree by
stz_gb300/build.py).  There is no fallback: if the library is missing or
fails to load, every call raises.
"""
import ctypes
import os

from .params import StzParams

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libstzg.so")

STZG_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "CUDA error",
          4: "multigrid did not converge", 5: "NaN residual", 6: "plastic sub-step cap reached",
          7: "no usable GPU"}

FP64 = 0
MIXED = 1
TOL_REFERENCE = 0
TOL_RELATIVE = 1
ADV_AUTO = 0
ADV_FP64 = 1
ADV_SPLIT = 2

# Every symbol include/stzg.h declares.
EXPORTS = [
    "stzg_default_options", "stzg_strerror", "stzg_last_message", "stzg_create", "stzg_destroy",
    "stzg_set_state", "stzg_init_fields", "stzg_chi_bicubic", "stzg_set_field", "stzg_get_field", "stzg_set_time", "stzg_get_time",
    "stzg_step_qs", "stzg_advection_step", "stzg_projection_step", "stzg_avg_iters",
    "stzg_mg_solve", "stzg_mg_vcycle", "stzg_mg_l2_error", "stzg_mg_levels", "stzg_mg_stencil",
    "stzg_l2_comparison", "stzg_random_chi", "stzg_upload", "stzg_download", "stzg_time_kernel",
    "stzg_set_mg_persistent", "stzg_get_mg_persistent", "stzg_residual_norms_noalloc",
    "stzg_c_field_pack", "stzg_c_field_unpack",
    "stzg_batch_create", "stzg_batch_destroy", "stzg_batch_size", "stzg_batch_sim", "stzg_batch_set_tuning",
    "stzg_batch_autotune", "stzg_batch_get_tuning", "stzg_batch_run",
    "stzg_adjoint_forward", "stzg_adjoint_backward",
    "stzg_step_direct", "stzg_advance_direct",
    "stzg_output_field", "stzg_write_frame", "stzg_qs_measure", "stzg_tractions", "stzg_compute_strain",
    "stzg_step_qs_host",
]


class StzgOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("tol_mode", ctypes.c_int), ("tol", ctypes.c_double),
                ("track_plastic", ctypes.c_int), ("device", ctypes.c_int), ("inner_cycles", ctypes.c_int),
                ("use_graphs", ctypes.c_int), ("extrapolate", ctypes.c_int),
                ("substep_cap", ctypes.c_int), ("advection", ctypes.c_int), ("reserved", ctypes.c_int * 5)]


class StzgStats(ctypes.Structure):
    _fields_ = [("vcycles", ctypes.c_long), ("extra_vcycles", ctypes.c_long), ("solves", ctypes.c_long),
                ("refinements", ctypes.c_long), ("checks", ctypes.c_long), ("last_error", ctypes.c_double),
                ("seconds", ctypes.c_double), ("substeps_max", ctypes.c_long),
                ("kernel_launches", ctypes.c_long)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StzgBatchStats(ctypes.Structure):
    _fields_ = [("instances", ctypes.c_long), ("steps", ctypes.c_long), ("cell_steps", ctypes.c_long),
                ("vcycles", ctypes.c_long), ("passes", ctypes.c_long), ("failed", ctypes.c_long),
                ("seconds", ctypes.c_double), ("graph_kernels", ctypes.c_long), ("kernel_launches", ctypes.c_long)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StzgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_P = ctypes.POINTER(ctypes.c_double)
_lib = None


def load(path=None):
    """Loads libstzg.so and declares the ABI.  Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    V = ctypes.c_void_p
    I = ctypes.c_int
    D = ctypes.c_double
    decl = {
        "stzg_default_options": (None, [ctypes.POINTER(StzgOptions)]),
        "stzg_strerror": (ctypes.c_char_p, [I]),
        "stzg_last_message": (ctypes.c_char_p, []),
        "stzg_create": (I, [ctypes.POINTER(StzParams), ctypes.POINTER(StzgOptions), ctypes.POINTER(V)]),
        "stzg_destroy": (I, [V]),
        "stzg_set_state": (I, [V, _P]),
        "stzg_init_fields": (I, [V, I, D, D]),
        "stzg_chi_bicubic": (I, [V, I, I, _P, D, D]),
        "stzg_set_field": (I, [V, I, _P]),
        "stzg_get_field": (I, [V, I, _P]),
        "stzg_set_time": (I, [V, D]),
        "stzg_get_time": (I, [V, _P]),
        "stzg_step_qs": (I, [V, D, I, ctypes.POINTER(StzgStats)]),
        "stzg_advection_step": (I, [V, D]),
        "stzg_projection_step": (I, [V, D, ctypes.POINTER(StzgStats)]),
        "stzg_avg_iters": (I, [V, _P]),
        "stzg_mg_solve": (I, [V, D, _P, _P, ctypes.POINTER(I)]),
        "stzg_mg_vcycle": (I, [V, D, _P, _P]),
        "stzg_mg_l2_error": (I, [V, D, _P, _P, _P]),
        "stzg_mg_levels": (I, [V, D, ctypes.POINTER(I), ctypes.POINTER(I)]),
        "stzg_mg_stencil": (I, [V, D, I, _P]),
        "stzg_l2_comparison": (I, [V, V, _P]),
        "stzg_random_chi": (I, [I, I, D, D, D, D, ctypes.c_ulonglong, _P]),
        "stzg_upload": (I, [V, ctypes.POINTER(ctypes.c_void_p)]),
        "stzg_download": (I, [V, ctypes.POINTER(ctypes.c_void_p)]),
        "stzg_time_kernel": (I, [V, D, I, I, _P]),
        "stzg_set_mg_persistent": (I, [V, I]),
        "stzg_c_field_pack": (I, [V, I, I, ctypes.POINTER(_P)]),
        "stzg_c_field_unpack": (I, [ctypes.POINTER(_P), I, I, V]),
        "stzg_get_mg_persistent": (I, [V, ctypes.POINTER(I)]),
        "stzg_residual_norms_noalloc": (I, [ctypes.POINTER(StzParams), D, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p]),
        "stzg_batch_create": (I, [I, ctypes.POINTER(StzParams), ctypes.POINTER(StzgOptions), ctypes.POINTER(V)]),
        "stzg_batch_destroy": (I, [V]),
        "stzg_batch_size": (I, [V, ctypes.POINTER(I)]),
        "stzg_batch_sim": (I, [V, I, ctypes.POINTER(V)]),
        "stzg_batch_set_tuning": (I, [V, I, I, I, ctypes.c_long, I]),
        "stzg_batch_autotune": (I, [V, D, I]),
        "stzg_batch_get_tuning": (I, [V, I, I, ctypes.POINTER(I), ctypes.POINTER(ctypes.c_long), ctypes.POINTER(I)]),
        "stzg_batch_run": (I, [V, D, I, ctypes.POINTER(StzgBatchStats)]),
        "stzg_adjoint_forward": (I, [V, D, I, I, _P, _P]),
        "stzg_adjoint_backward": (I, [V, D, _P, _P]),
        "stzg_step_direct": (I, [V, D, I, ctypes.POINTER(StzgStats)]),
        "stzg_advance_direct": (I, [V, D, D, ctypes.POINTER(ctypes.c_long)]),
        "stzg_output_field": (I, [V, I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_long)]),
        "stzg_write_frame": (I, [V, ctypes.c_char_p, I, ctypes.c_uint, _P]),
        "stzg_qs_measure": (I, [V, I, _P, _P]),
        "stzg_tractions": (I, [V, _P]),
        "stzg_compute_strain": (I, [V, _P]),
        "stzg_step_qs_host": (I, [V, D, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                  ctypes.POINTER(StzgStats)]),
    }
    for name, (res, args) in decl.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != STZG_OK:
        msg = load().stzg_last_message().decode(errors="replace")
        raise StzgError(status, msg)


def default_options(**kw):
    o = StzgOptions()
    load().stzg_default_options(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o
