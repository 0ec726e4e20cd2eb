"""Host-side mirror of the reference's general multigrid template
tgmg<S,double,double> (esim/tgmg/tgmg.hh:286-495) and of its poisson_fd
problem class (esim/tgmg/poisson_fd.{hh,cc}) over the C ABI in
include/stzg_tgmg.h.  The hierarchy, the cycles and the convergence checks run
on the GPU (libstzg.so); there is no CPU path.

As in the reference, a solver works on the problem's own b and z arrays: each
solve copies b and z to the device and z back.  ``Tgmg.solve_*`` return True
on convergence and False where the reference returns false (the predictor's
threshold exceeded); other failures raise.
"""
import ctypes

import numpy as np

from . import _lib

# Every symbol include/stzg_tgmg.h declares.
EXPORTS = [
    "stzg_tgmg_predict_init", "stzg_tgmg_create", "stzg_tgmg_create_block", "stzg_tgmg_set_operator",
    "stzg_tgmg_set_precision", "stzg_tgmg_solve_checked",
    "stzg_tgmg_destroy", "stzg_tgmg_set_b", "stzg_tgmg_get_b",
    "stzg_tgmg_set_z", "stzg_tgmg_get_z", "stzg_tgmg_device_arrays", "stzg_tgmg_clear_z", "stzg_tgmg_solve", "stzg_tgmg_solve_fixed",
    "stzg_tgmg_iterate", "stzg_tgmg_l2_error", "stzg_tgmg_levels", "stzg_tgmg_stencil", "stzg_tgmg_last_timing",
    "stzg_poisson_fd",
]

JACOBI, GAUSS_SEIDEL, SOR, FMG, VCYCLE, SYM_VCYCLE = range(6)
# (per_loop, max_loops) of the fixed-batch solves, tgmg_config.hh:6-19
FIXED_LOOPS = {JACOBI: (100, 400), GAUSS_SEIDEL: (20, 2000), SOR: (20, 1000), FMG: (2, 1000), VCYCLE: (4, 1000)}

_P = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)


class Predict(ctypes.Structure):
    """tgmg_predict (tgmg_predict.hh:6-33): the adaptive iteration count."""
    _fields_ = [("mult", ctypes.c_int), ("decay", ctypes.c_int), ("max_thresh", ctypes.c_int),
                ("extra_iters", ctypes.c_int), ("lim", ctypes.c_int), ("solves", ctypes.c_int),
                ("vcount", ctypes.c_int)]

    def __init__(self):
        super().__init__()
        load().stzg_tgmg_predict_init(ctypes.byref(self))

    def avg_iters(self):
        """Average count per solve since the last call, then reset (NaN
        before any solve, as the reference's float division gives)."""
        ans = float(self.vcount) / self.solves if self.solves else float("nan")
        self.solves = self.vcount = 0
        return ans


def load():
    lib = _lib.load()
    if getattr(lib, "_tgmg_declared", False):
        return lib
    V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    PP = ctypes.POINTER(Predict)
    decl = {
        "stzg_tgmg_predict_init": (None, [PP]),
        "stzg_tgmg_create": (I, [I, I, I, I, _P, I, _IP, D, I, ctypes.POINTER(V)]),
        "stzg_tgmg_create_block": (I, [I, I, I, I, I, _P, I, _IP, D, I, ctypes.POINTER(V)]),
        "stzg_tgmg_set_operator": (I, [V, _P, I, _IP]),
        "stzg_tgmg_set_precision": (I, [V, I]),
        "stzg_tgmg_solve_checked": (I, [V, I, I, I, D, I, I, I, _IP, _P]),
        "stzg_tgmg_destroy": (I, [V]),
        "stzg_tgmg_set_b": (I, [V, _P]),
        "stzg_tgmg_get_b": (I, [V, _P]),
        "stzg_tgmg_set_z": (I, [V, _P]),
        "stzg_tgmg_get_z": (I, [V, _P]),
        "stzg_tgmg_device_arrays": (I, [V, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]),
        "stzg_tgmg_clear_z": (I, [V]),
        "stzg_tgmg_solve": (I, [V, I, PP, D, I, I, I, _IP, _P]),
        "stzg_tgmg_solve_fixed": (I, [V, I, I, I, D, I, I, I, _IP, _P]),
        "stzg_tgmg_iterate": (I, [V, I, I, D, I, I, I]),
        "stzg_tgmg_l2_error": (I, [V, _P]),
        "stzg_tgmg_levels": (I, [V, _IP, _IP]),
        "stzg_tgmg_stencil": (I, [V, I, _P]),
        "stzg_tgmg_last_timing": (I, [V, _P, ctypes.POINTER(ctypes.c_long)]),
        "stzg_poisson_fd": (I, [I, I, D, D, D, D, _P, _IP, _P]),
    }
    for name, (res, args) in decl.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._tgmg_declared = True
    return lib


def _dp(a):
    return a.ctypes.data_as(_P)


class Problem:
    """A problem class in the sense of tgmg's template arguments S, V, M: an
    m x n grid with periodicity flags, its 9-point operator as a table of
    stencils (dl dc dr cl cc cr ul uc ur; scalars, or row-major 2x2 blocks when
    block = 2) with a stencil index per point, the squared residual threshold
    acc, and the arrays b and z (n rows of m, times block components)."""

    def __init__(self, m, n, table, cls, acc, x_prd=False, y_prd=False, block=1):
        self.m, self.n, self.block = int(m), int(n), int(block)
        self.x_prd, self.y_prd = bool(x_prd), bool(y_prd)
        self.table = np.ascontiguousarray(np.asarray(table, dtype=np.float64).reshape(-1, 9 * self.block ** 2))
        self.cls = np.ascontiguousarray(np.asarray(cls, dtype=np.int32).reshape(self.n, self.m))
        self.acc = float(acc)
        shape = (self.n, self.m) if self.block == 1 else (self.n, self.m, self.block)
        self.b = np.zeros(shape)
        self.z = np.zeros(shape)


class PoissonFD(Problem):
    """poisson_fd (poisson_fd.hh:7-61, poisson_fd.cc:12-39): the 5-point
    Laplacian on m x n grid points spanning [ax,bx] x [ay,by], Dirichlet edges,
    acc = tgmg_accuracy(hcc, 1e4)."""

    def __init__(self, m, n, ax, bx, ay, by):
        lib = load()
        table = np.zeros(18)
        cls = np.zeros(m * n, dtype=np.int32)
        acc = ctypes.c_double()
        _lib.check(lib.stzg_poisson_fd(m, n, ax, bx, ay, by, _dp(table), cls.ctypes.data_as(_IP),
                                       ctypes.byref(acc)))
        super().__init__(m, n, table, cls, acc.value)
        self.ax, self.ay = float(ax), float(ay)
        self.dx = (bx - ax) / (m - 1)
        self.dy = (by - ay) / (n - 1)
        self.hcc, self.hxx, self.hyy = table[4], table[3], table[1]
        self.hcc_inv = 1. / self.hcc

    def gaussian_source_term(self, gx, gy, r, amp):
        """poisson_fd::gaussian_source_term (poisson_fd.cc:30-39): x advances
        by repeated addition of dx along each row, as in the reference loop."""
        lam = -0.5 / (r * r)
        xs = np.add.accumulate(np.concatenate(([self.ax - gx], np.full(self.m - 1, self.dx))))
        for j in range(self.n):
            y = self.ay - gy + self.dy * j
            self.b[j, :] = amp * np.exp(lam * (xs * xs + y * y))


class Tgmg:
    """tgmg<S,double,double> on the GPU for a Problem (tgmg.in.cc:11-33):
    the hierarchy and its Galerkin operators are built at construction
    (tgmg::setup, tgmg.hh:331-335)."""

    def __init__(self, q, device=0):
        self.lib = load()
        self.q = q
        self.verbose = 0
        h = ctypes.c_void_p()
        _lib.check(self.lib.stzg_tgmg_create_block(q.m, q.n, int(q.x_prd), int(q.y_prd), getattr(q, "block", 1),
                                                   _dp(q.table), q.table.shape[0], q.cls.ctypes.data_as(_IP), q.acc,
                                                   device, ctypes.byref(h)))
        self.h = h

    def set_operator(self, table, cls=None, keep_classes=False):
        """New stencil values on the same grid (qs_multi::init + setup).
        keep_classes: the class map stays the solver's last one and is not
        passed (the same number of stencils is then required)."""
        q = self.q
        table = np.ascontiguousarray(np.asarray(table, dtype=np.float64).reshape(-1, q.table.shape[1]))
        if keep_classes:
            _lib.check(self.lib.stzg_tgmg_set_operator(self.h, _dp(table), table.shape[0], None))
            q.table = table
            return
        q.table = table
        if cls is not None:
            q.cls = np.ascontiguousarray(np.asarray(cls, dtype=np.int32).reshape(q.n, q.m))
        _lib.check(self.lib.stzg_tgmg_set_operator(self.h, _dp(q.table), q.table.shape[0],
                                                   q.cls.ctypes.data_as(_IP)))

    def set_precision(self, mixed):
        """mixed: V-cycle solves and iterations run as refinement passes (an
        FP32 V-cycle on the FP64 residual, the correction added in FP64)."""
        _lib.check(self.lib.stzg_tgmg_set_precision(self.h, 1 if mixed else 0))

    def close(self):
        if getattr(self, "h", None):
            self.lib.stzg_tgmg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup(self):
        """The hierarchy was set up when the handle was created."""

    # -- data movement ------------------------------------------------------
    def _push(self):
        b = np.ascontiguousarray(self.q.b, dtype=np.float64)
        z = np.ascontiguousarray(self.q.z, dtype=np.float64)
        _lib.check(self.lib.stzg_tgmg_set_b(self.h, _dp(b)))
        _lib.check(self.lib.stzg_tgmg_set_z(self.h, _dp(z)))

    def _pull(self):
        z = np.empty(self.q.z.shape)
        _lib.check(self.lib.stzg_tgmg_get_z(self.h, _dp(z)))
        self.q.z[...] = z

    def clear_z(self):
        self.q.z[...] = 0

    # -- solves -------------------------------------------------------------
    def _solve(self, kind, tp, omega=1.0, cyc_down=1, cyc_up=1, hcyc_bottom=10):
        self._push()
        it, l2 = ctypes.c_int(), ctypes.c_double()
        if tp is None:
            per, loops = FIXED_LOOPS[kind]
            st = self.lib.stzg_tgmg_solve_fixed(self.h, kind, per, loops, omega, cyc_down, cyc_up, hcyc_bottom,
                                                ctypes.byref(it), ctypes.byref(l2))
        else:
            st = self.lib.stzg_tgmg_solve(self.h, kind, ctypes.byref(tp), omega, cyc_down, cyc_up, hcyc_bottom,
                                          ctypes.byref(it), ctypes.byref(l2))
        self._pull()
        self.iterations, self.residual = it.value, l2.value
        if st == 4:  # not converged: the reference returns false
            return False
        _lib.check(st)
        return True

    def solve_v_cycle_checked(self, max_iters=2048, extra_iters=1, cyc_down=1, cyc_up=1, hcyc_bottom=10):
        """V-cycles until l2_error < acc, tested before the first and after
        each, then extra_iters more (not in the reference)."""
        self._push()
        it, l2 = ctypes.c_int(), ctypes.c_double()
        st = self.lib.stzg_tgmg_solve_checked(self.h, VCYCLE, max_iters, extra_iters, 1.0, cyc_down, cyc_up,
                                              hcyc_bottom, ctypes.byref(it), ctypes.byref(l2))
        self._pull()
        self.iterations, self.residual = it.value, l2.value
        if st == 4:
            return False
        _lib.check(st)
        return True

    def solve_v_cycle(self, tp=None, cyc_down=1, cyc_up=1, hcyc_bottom=10):
        return self._solve(VCYCLE, tp, 1.0, cyc_down, cyc_up, hcyc_bottom)

    def solve_sym_v_cycle(self, tp, cyc_down=1, cyc_up=1, hcyc_bottom=10):
        return self._solve(SYM_VCYCLE, tp, 1.0, cyc_down, cyc_up, hcyc_bottom)

    def solve_full_multigrid(self, tp=None, cyc_down=1, cyc_up=1, hcyc_bottom=10):
        return self._solve(FMG, tp, 1.0, cyc_down, cyc_up, hcyc_bottom)

    def solve_jacobi(self, tp=None):
        return self._solve(JACOBI, tp)

    def solve_gauss_seidel(self, tp=None):
        return self._solve(GAUSS_SEIDEL, tp)

    def solve_sor(self, omega, tp=None):
        return self._solve(SOR, tp, omega)

    # -- single iterations ----------------------------------------------------
    def _iterate(self, kind, count=1, omega=1.0, cyc_down=1, cyc_up=1, hcyc_bottom=10):
        self._push()
        _lib.check(self.lib.stzg_tgmg_iterate(self.h, kind, count, omega, cyc_down, cyc_up, hcyc_bottom))
        self._pull()

    def v_cycle(self, cyc_down=1, cyc_up=1, hcyc_bottom=10, symmetric=False):
        self._iterate(SYM_VCYCLE if symmetric else VCYCLE, 1, 1.0, cyc_down, cyc_up, hcyc_bottom)

    def jacobi(self):
        self._iterate(JACOBI)

    def gauss_seidel(self):
        self._iterate(GAUSS_SEIDEL)

    def sor(self, omega):
        self._iterate(SOR, 1, omega)

    def l2_error(self):
        self._push()
        e = ctypes.c_double()
        _lib.check(self.lib.stzg_tgmg_l2_error(self.h, ctypes.byref(e)))
        return e.value

    # -- hierarchy ------------------------------------------------------------
    def levels(self):
        nl = ctypes.c_int()
        dims = np.zeros(2 * 17, dtype=np.int32)
        _lib.check(self.lib.stzg_tgmg_levels(self.h, ctypes.byref(nl), dims.ctypes.data_as(_IP)))
        return [(int(dims[2 * k]), int(dims[2 * k + 1])) for k in range(nl.value)]

    def stencil(self, level):
        """Galerkin stencils of coarse level `level` (1 = first child), shape
        (n, m, 10) as tgmg_level::s, or (n, m, 10, 2, 2) for 2x2 blocks."""
        m, n = self.levels()[level]
        B = getattr(self.q, "block", 1)
        out = np.empty((n, m, 10) if B == 1 else (n, m, 10, B, B))
        _lib.check(self.lib.stzg_tgmg_stencil(self.h, level, _dp(out)))
        return out

    def last_timing(self):
        ms, k = ctypes.c_double(), ctypes.c_long()
        _lib.check(self.lib.stzg_tgmg_last_timing(self.h, ctypes.byref(ms), ctypes.byref(k)))
        return ms.value, k.value
