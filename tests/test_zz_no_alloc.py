"""The no-allocation entry point stzg_residual_norms_noalloc.

It serves callers that cannot let this library call cudaMalloc (an
application allocator that owns the device memory, a fixed memory budget, a
thread that must not stall the GPU): its reduction scratch is a static
device array.  It is checked through the C ABI against the allocating path
(stzg_mg_l2_error on a handle, which reduces through the handle's own scratch)
and against the CPU oracle's residual sum (mds, tgmg.in.cc:55-64) on two
calls in a row with different inputs, so the second call also shows that
nothing left in the shared array leaks into the next result.  This file
is collected last so that a run stopping at its first failure has run every
other test.
"""
import ctypes

import numpy as np
import pytest

from oracle.bind import OracleSim
from stz_gb300 import _lib
from stz_gb300.params import simple_shear
from stz_gb300.shear_sim import ShearSim

pytestmark = pytest.mark.gpu


def test_noalloc_residual_norms_match_allocating_path():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    N = 96
    P = simple_shear(N)
    dt = 0.01
    chi = np.full((N, N), 600 / 21000.0)
    sim = ShearSim(P, chi)
    oracle = OracleSim(P, chi)
    nodes = N * (N + 1)
    rng = np.random.default_rng(17)
    dev = torch.device("cuda", 0)
    for call in range(2):
        src = rng.standard_normal((N + 1, N, 2)) * (10.0 ** call)
        vel = rng.standard_normal((N + 1, N, 2)) * 1e-3
        z = torch.from_numpy(vel.copy()).to(dev)
        b = torch.from_numpy(src.copy()).to(dev)
        out = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = lib.stzg_residual_norms_noalloc(ctypes.byref(P), dt, z.data_ptr(), b.data_ptr(), out.data_ptr(), None)
        assert st == 0, lib.stzg_last_message()
        torch.cuda.synchronize()
        r2, b2 = out.cpu().numpy()
        mean_sq = sim.mg_l2_error(dt, src, vel)  # allocating path: sum/nodes
        assert r2 == pytest.approx(mean_sq * nodes, rel=1e-12)
        assert b2 == pytest.approx(float(np.sum(src ** 2)), rel=1e-12)
        o_r2, o_b2 = oracle.mg_residual_sqnorms(dt, src, vel)
        assert r2 == pytest.approx(o_r2, rel=1e-12)
        assert b2 == pytest.approx(o_b2, rel=1e-12)


def test_noalloc_rejects_oversized_grid():
    lib = _lib.load()
    P = simple_shear(4096)  # 4096 x 4097 nodes > 8,388,608
    st = lib.stzg_residual_norms_noalloc(ctypes.byref(P), 0.01, ctypes.c_void_p(16), ctypes.c_void_p(16),
                                         ctypes.c_void_p(16), None)
    assert st == 1
    assert "too large" in lib.stzg_last_message().decode()
