"""The reference's own driver programs compile and link, unmodified, against
the drop-in (include/dropin/shear_sim.hh over include/stzg_shear_sim.hh and
libstzg.so).

Every driver of esim/sb/main that uses shear_sim is read where it lies and
compiled from standard input, so that the reference's own shear_sim.hh
beside it is not found first; the reference's common.cc (safe_fopen,
fatal_error) is compiled from its tree as the drivers' own helper.  Nothing
runs: that needs a GPU (tests/test_gpu_cpp_dropin.py runs a driver written the
same way).  Skipped where the reference tree is absent, as on the GPU host.
"""
import os
import subprocess

import pytest

from oracle.bind import reference_root

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVERS = ["shear_random", "shear_compare", "shear_mcompare", "shear_runs", "shear_small", "shear_test",
           "shear_test2", "shear_test3"]
LIB = os.path.join(ROOT, "stz_gb300", "_build")


@pytest.fixture(scope="module")
def main_dir():
    root = reference_root()
    if root is None:
        pytest.skip("reference tree not present")
    d = os.path.join(root, "esim", "sb", "main")
    if not os.path.isdir(d):
        pytest.skip("esim/sb/main not present")
    return d


def compile_driver(src, obj, main_dir):
    with open(src) as f:
        code = f.read()
    cmd = ["g++", "-std=c++17", "-fopenmp", "-c", "-x", "c++", "-", "-o", obj,
           "-I", os.path.join(ROOT, "include", "dropin"), "-I", os.path.join(ROOT, "include"), "-I", main_dir]
    return subprocess.run(cmd, input=code, capture_output=True, text=True)


@pytest.mark.parametrize("name", DRIVERS)
def test_reference_driver_compiles_against_dropin(name, main_dir, tmp_path):
    r = compile_driver(os.path.join(main_dir, name + ".cc"), str(tmp_path / (name + ".o")), main_dir)
    assert r.returncode == 0, r.stderr


def test_reference_drivers_link_against_libstzg(main_dir, tmp_path):
    if not os.path.exists(os.path.join(LIB, "libstzg.so")):
        pytest.skip("libstzg.so not built")
    common = str(tmp_path / "common.o")
    r = subprocess.run(["g++", "-c", os.path.join(main_dir, "common.cc"), "-o", common], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    for name in ("shear_random", "shear_compare", "shear_test"):
        obj = str(tmp_path / (name + ".o"))
        r = compile_driver(os.path.join(main_dir, name + ".cc"), obj, main_dir)
        assert r.returncode == 0, r.stderr
        r = subprocess.run(["g++", "-fopenmp", obj, common, "-o", str(tmp_path / name), "-L", LIB, "-lstzg"],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
