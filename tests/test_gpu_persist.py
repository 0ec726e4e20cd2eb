"""The persistent coarse multigrid kernel: the FP32 V-cycle's levels of at
most 512 columns and its single-block tail in one cooperative launch with
grid barriers between the level phases.  The arithmetic per point is that of
the per-level kernels, so steps agree bit for bit with the per-level schedule
(which the parity tests pin to the CPU oracle).  The kernel is off by default
(slower than the per-level launches on GB300) and switched on per handle."""
import numpy as np
import pytest

from stz_gb300 import _lib
from stz_gb300.params import simple_shear
from stz_gb300.shear_sim import ShearSim, random_chi

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "p", "q", "s", "tau", "chi", "X", "Y")


def _pair(m, n, steps, seed, **kw):
    P = simple_shear(m, n) if n != m else simple_shear(m)
    chi = random_chi(m, n, 6, 600.0, 40.0, P.TZ, seed)
    out = []
    for persist in (True, False):
        g = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-10, extrapolate=1, **kw)
        g.mg_persistent = persist
        g.steps(0.01, steps)
        assert g.mg_persistent == persist  # the levels qualify at these sizes
        out.append((g.fields(), g.cycles))
        g.close()
    return out


@pytest.mark.parametrize("m,n", [(256, 256), (512, 512), (384, 320), (640, 384)])
def test_persistent_matches_per_level_schedule(m, n):
    (a, ca), (b, cb) = _pair(m, n, 4, 3)
    assert ca == cb
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), f


def test_persistent_off_by_default_and_switchable():
    P = simple_shear(512)
    chi = random_chi(512, 512, 6, 600.0, 40.0, P.TZ, 1)
    g = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-10)
    assert not g.mg_persistent
    g.steps(0.01, 1)
    assert not g.mg_persistent
    g.mg_persistent = True
    g.steps(0.01, 1)
    assert g.mg_persistent
    g.mg_persistent = False
    assert not g.mg_persistent
    g.close()
    f64 = ShearSim(simple_shear(64), random_chi(64, 64, 4, 600.0, 30.0, P.TZ, 1), precision=_lib.FP64)
    with pytest.raises(_lib.StzgError):
        f64.mg_persistent = True
    f64.close()


def test_persistent_barrier_time_limit():
    """A barrier that can never complete (arrival count set out of reach):
    every block gives up after its bounded wait, the step reports
    STZG_ECUDA, and the context stays usable for a new handle."""
    P = simple_shear(256)
    chi = random_chi(256, 256, 6, 600.0, 40.0, P.TZ, 2)
    g = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-10)
    g.mg_persistent = True
    g.steps(0.01, 1)
    g.lib.stzg_set_mg_persistent(g.h, 2)
    with pytest.raises(_lib.StzgError) as e:
        g.steps(0.01, 1)
    assert e.value.status == 3  # STZG_ECUDA
    assert "barrier" in str(e.value)
    g.close()
    h = ShearSim(P, chi, precision=_lib.MIXED, tol_mode=_lib.TOL_RELATIVE, tol=1e-10)
    h.mg_persistent = True
    h.steps(0.01, 2)
    assert h.mg_persistent
    h.close()
