"""The C++ drop-in (include/dropin/shear_sim.hh over include/stzg_shear_sim.hh),
compiled into a small driver written like the reference's drivers (law
object, constructor arguments, sim.time, solve / solve_quasistatic with frame
files, tractions, qs_measure), against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from oracle.bind import OracleSim
from parity import group_errors
from stz_gb300.params import plastic_shear

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_driver(tmp_path, *args):
    exe = tmp_path / "dropin"
    lib = os.path.join(ROOT, "stz_gb300", "_build")
    if not exe.exists():
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-I", os.path.join(ROOT, "include", "dropin"),
                               "-I", os.path.join(ROOT, "include"),
                               os.path.join(ROOT, "tests", "cpp", "dropin_main.cc"), "-o", str(exe),
                               "-L", lib, "-lstzg", f"-Wl,-rpath,{lib}"])
    out = tmp_path / "fields.bin"
    frames = tmp_path / "frames"
    frames.mkdir(exist_ok=True)
    r = subprocess.run([str(exe), str(out), args[0], str(frames), *args[1:]], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return r, read_fields(out)


def read_fields(out):
    N = 32
    raw = np.fromfile(out)
    cells, nodes = N * (N + 2), N * (N + 1)
    sizes = [N * N] + [cells] * 5 + [nodes] * 4 + [N * N]
    parts = np.split(raw, np.cumsum(sizes)[:-1])
    chi0 = parts[0].reshape(N, N)
    names = ["p", "q", "s", "tau", "chi", "X", "Y", "u", "v", "eps_pl"]
    got = {k: v for k, v in zip(names, parts[1:])}
    for k in ("p", "q", "s", "tau", "chi"):
        got[k] = got[k].reshape(N + 2, N)
    for k in ("X", "Y", "u", "v"):
        got[k] = got[k].reshape(N + 1, N)
    got["eps_pl"] = got["eps_pl"].reshape(N, N)
    return chi0, got


def test_cpp_dropin_matches_oracle(tmp_path):
    N = 32
    r, (chi0, got) = run_driver(tmp_path, "10")
    P = plastic_shear(N)
    o = OracleSim(P, chi0)
    o.set_tolerance(0, 10.0)
    o.steps(0.01, 80)
    err = group_errors(o.fields(), got, N)
    assert max(err.values()) < 1e-9, err
    assert "avg_iters" in r.stdout
    # sim.time is the reference's public member: 80 steps of 0.01
    assert abs(float(r.stdout.split()[1]) - 0.8) < 1e-12


def test_cpp_dropin_quasistatic_frames(tmp_path):
    """shear_sim::solve_quasistatic (two frames of 40 steps) writes frames
    0, 1, 2 of the reference's five fields and follows the oracle."""
    N = 32
    r, (chi0, got) = run_driver(tmp_path, "10", "frames")
    P = plastic_shear(N)
    o = OracleSim(P, chi0)
    o.set_tolerance(0, 10.0)
    o.steps(0.01, 80)
    err = group_errors(o.fields(), got, N)
    assert max(err.values()) < 1e-9, err
    for k in range(3):
        for f in ("p", "tem", "dev", "X", "Y"):
            assert (tmp_path / "frames" / f"{f}.{k}").stat().st_size > 0
    assert "# Output frame 2 [40," in r.stdout


def test_cpp_dropin_explicit_solve(tmp_path):
    """shear_sim::solve (explicit steps of dx^2 tmult, two frames) through the
    C++ mirror, against the oracle's frame loop."""
    N = 32
    r, (chi0, got) = run_driver(tmp_path, "10", "direct")
    P = plastic_shear(N)
    o = OracleSim(P, chi0)
    dt = (2.0 / N) ** 2 * 0.5
    o.advance_direct(dt, 0.05)
    o.advance_direct(dt, 0.1)
    err = group_errors(o.fields(), got, N)
    assert max(err.values()) < 1e-10, err
