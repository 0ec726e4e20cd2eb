"""Initial states and l2_comparison on the GPU against fixtures the
reference produced (tests/golden/make_golden.py).

* stzg_init_fields (shear_sim::init_fields, shear_sim.cc:60-114) and
  stzg_chi_bicubic (shear_sim::initialize_chi_bicubic, shear_sim.cc:832-909):
  the initial state equals the reference's to rounding, and quasi-static
  steps from it follow the reference.
* stzg_l2_comparison (shear_sim::l2_comparison, shear_sim.cc:460-502): on
  two handles that hold the fixture's two runs exactly it gives the
  reference's numbers to rounding; on the GPU's own explicit and
  quasi-static runs from the fixture's chi it follows the reference's runs.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from parity import group_errors
from stz_gb300 import _lib
from stz_gb300.shear_sim import ShearSim

pytestmark = pytest.mark.gpu

INIT_FIELDS = ("u", "v", "p", "q", "s", "tau", "chi", "X", "Y", "ddev")


@pytest.mark.parametrize("name", golden_names("init"))
def test_initial_states_match_reference(name):
    P, meta, ref = load_golden(name)
    g = ShearSim(P, tol_mode=_lib.TOL_RELATIVE, tol=1e-13)
    setup = meta["setup"]
    if setup[0] == "init":
        g.init_fields(*setup[1:])
    else:
        g.initialize_chi_bicubic(ref["bicubic_arr"], setup[2], setup[3])
    got = g.fields()
    for k in INIT_FIELDS:
        a, b = ref[k + "0"], got[k]
        if k == "chi" and setup[0] == "bicubic":
            a, b = a[1:-1], b[1:-1]  # the reference leaves the ghost rows as they were
        assert np.abs(a - b).max() <= 1e-15 * max(np.abs(a).max(), 1.0), (name, k)
    assert g.time == 0.0
    g.steps(meta["dt"], meta["steps"])
    err = group_errors(ref, g.fields(), P.n)
    assert max(err.values()) < 1e-10, (name, err)
    g.close()


def holding(P, ref, prefix):
    """A handle holding one of the fixture's runs field for field."""
    g = ShearSim(P, ref["chi0"])
    for k in ("p", "q", "s", "tau", "chi", "X", "Y", "u", "v"):
        g.set(k, ref[prefix + k])
    return g


@pytest.mark.parametrize("name", golden_names("l2"))
def test_l2_comparison_on_reference_fields(name):
    P, meta, ref = load_golden(name)
    a, b = holding(P, ref, "direct_"), holding(P, ref, "qs_")
    np.testing.assert_allclose(a.l2_comparison(b), ref["l2"][-1], rtol=1e-12, atol=1e-300)
    np.testing.assert_array_equal(a.l2_comparison(a), np.zeros(4))
    a.close()
    b.close()


@pytest.mark.parametrize("name", golden_names("l2"))
def test_l2_comparison_of_gpu_runs(name):
    """The shear_compare workflow: an explicit run (frame loop of
    shear_sim::solve) and a quasi-static run advanced to the same frame
    times, compared after every frame."""
    P, meta, ref = load_golden(name)
    d = ShearSim(P, ref["chi0"])
    q = ShearSim(P, ref["chi0"], tol_mode=_lib.TOL_RELATIVE, tol=1e-13)
    got = [d.l2_comparison(q)]
    t_prev = 0.0
    for t in meta["frames"]:
        d.advance_direct(meta["dt"], t)
        q.steps((t - t_prev) / meta["qs_steps"], meta["qs_steps"])
        t_prev = t
        got.append(d.l2_comparison(q))
    np.testing.assert_allclose(np.array(got), ref["l2"], rtol=1e-8, atol=1e-300)
    for prefix, sim in (("direct_", d), ("qs_", q)):
        err = group_errors({k[len(prefix):]: v for k, v in ref.items() if k.startswith(prefix)}, sim.fields(), P.n)
        assert max(err.values()) < 1e-10, (name, prefix, err)
    d.close()
    q.close()
