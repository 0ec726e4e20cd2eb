"""Batches of independent simulations run in one CUDA graph (stzg_batch_*).

The reference runs one shear_sim per process; its UQ calibration harness
(esim/coord_transforms/simple_shear/pfn.py) launches one process per sample.
A Batch holds many simulations of possibly different grid sizes and advances
all of them with a single graph launch.
"""
import ctypes

import numpy as np

from . import _lib
from .params import StzParams, simple_shear
from .shear_sim import ShearSim, random_chi

SIZES = (64, 96, 128, 192, 256, 384, 512)


class Batch:
    def __init__(self, params, chis=None, *, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-10,
                 extrapolate=True, inner_cycles=0, device=0, track_plastic=True):
        lib = _lib.load()
        self.lib = lib
        self.params = [p.copy() for p in params]
        arr = (StzParams * len(params))(*self.params)
        self.options = _lib.default_options(precision=precision, tol_mode=tol_mode, tol=tol,
                                            extrapolate=int(extrapolate), inner_cycles=inner_cycles,
                                            device=device, track_plastic=int(track_plastic))
        h = ctypes.c_void_p()
        _lib.check(lib.stzg_batch_create(len(params), arr, ctypes.byref(self.options), ctypes.byref(h)))
        self.h = h
        self.stats = _lib.StzgBatchStats()
        self.views = []
        for k, p in enumerate(self.params):
            sh = ctypes.c_void_p()
            _lib.check(lib.stzg_batch_sim(h, k, ctypes.byref(sh)))
            self.views.append(ShearSim.view(sh, p))
        if chis is not None:
            for k, chi in enumerate(chis):
                self.views[k].set_state(chi)

    def __len__(self):
        return len(self.views)

    def sim(self, k):
        return self.views[k]

    def close(self):
        if getattr(self, "h", None):
            self.lib.stzg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, dt, nsteps):
        st = _lib.StzgBatchStats()
        _lib.check(self.lib.stzg_batch_run(self.h, float(dt), int(nsteps), ctypes.byref(st)))
        self.stats = st
        return st

    def set_tuning(self, m, n, inner, tail_limit=-1, fuse=1):
        _lib.check(self.lib.stzg_batch_set_tuning(self.h, m, n, inner, tail_limit, fuse))

    def autotune(self, dt, steps=4):
        _lib.check(self.lib.stzg_batch_autotune(self.h, float(dt), int(steps)))
        return {(p.m, p.n): self.tuning(p.m, p.n) for p in self.params}

    def tuning(self, m, n):
        i, t, f = ctypes.c_int(), ctypes.c_long(), ctypes.c_int()
        _lib.check(self.lib.stzg_batch_get_tuning(self.h, m, n, ctypes.byref(i), ctypes.byref(t), ctypes.byref(f)))
        return {"inner": i.value, "tail_limit": t.value, "fuse": f.value}


def batched_config(count=256, seed=2026):
    """The batched configuration: grids uniform over 64..512 squared, chi std
    U[10,50] K (mean 600 K, correlation length 4 cells), c0 U[0.2,0.6],
    chi_inf U[800,1000] K; simple shear at the reference-like wall speed."""
    rng = np.random.default_rng(seed)
    params, chis = [], []
    for k in range(count):
        N = int(rng.choice(SIZES))
        p = simple_shear(N, c0=float(rng.uniform(0.2, 0.6)), chi_inf_K=float(rng.uniform(800.0, 1000.0)))
        std = float(rng.uniform(10.0, 50.0))
        params.append(p)
        chis.append(random_chi(N, N, 4.0, 600.0, std, p.TZ, seed * 1000 + k))
    return params, chis
