import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)

GOLDEN = os.path.join(TESTS, "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path)")


def golden_names(kind="quasistatic"):
    """Fixture names of one kind: "quasistatic" (step_forward_quasistatic),
    "direct" (the explicit step_forward), "frames" (output and
    diagnostics of a quasi-static state), "tgmg" (the general multigrid on
    poisson_fd), "ct" (the step in sheared coordinates), "ct_tracers" (its
    Lagrangian tracers), "ct_direct" (its explicit step), "ct_bicubic" (its
    bicubic chi set-up), "ct_frames" (its frame files), "ct_l2t" (its
    l2_comparison_transform), "init" (the
    initial states of init_fields and initialize_chi_bicubic, then
    quasi-static steps), "l2" (l2_comparison of an explicit and a
    quasi-static run) or "coarse" (the coarse Galerkin operators of the
    quasi-static system)."""
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    prefix = {"direct": ("direct_",), "frames": ("frames_",), "tgmg": ("tgmg_",), "ct": ("ct_",),
              "ct_tracers": ("ct_tracers_",), "ct_direct": ("ctdirect_",), "ct_bicubic": ("ct_bicubic_",), "ct_frames": ("ct_frames_",), "ct_l2t": ("ct_l2t_",), "init": ("init_", "bicubic_"),
              "l2": ("l2cmp_",), "coarse": ("coarseops_",)}
    if kind == "ct":
        return [n for n in names
                if n.startswith("ct_") and not n.startswith(("ct_tracers_", "ct_bicubic_", "ct_frames_", "ct_l2t_"))]
    if kind in prefix:
        return [n for n in names if n.startswith(prefix[kind])]
    return [n for n in names if not any(n.startswith(p) for ps in prefix.values() for p in ps)]


def load_golden(name):
    from stz_gb300.params import StzParams
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    P = StzParams()
    for k, v in meta["params"].items():
        setattr(P, k, v)
    fields = {k: d[k] for k in d.files if k not in ("meta",)}
    return P, meta, fields


@pytest.fixture(params=golden_names())
def golden(request):
    return (request.param,) + load_golden(request.param)


@pytest.fixture(params=golden_names("direct"))
def golden_direct(request):
    return (request.param,) + load_golden(request.param)


@pytest.fixture(params=golden_names("frames"))
def golden_frames(request):
    return (request.param,) + load_golden(request.param)


def load_tgmg_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    return meta, {k: d[k] for k in d.files if k != "meta"}


@pytest.fixture(params=golden_names("tgmg"))
def golden_tgmg(request):
    return (request.param,) + load_tgmg_golden(request.param)
