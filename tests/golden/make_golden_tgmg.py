"""Regenerates the general-multigrid golden fixtures from the reference itself.

Run where the SURGroup/STZ tree is available (the tree oracle/build_ref.sh
resolves: STZ_REFERENCE_ROOT, else the recipe's default):

    python tests/golden/make_golden_tgmg.py

It builds oracle/_ref/libtgmgref.so (oracle/build_ref.sh: the reference's
esim/tgmg/poisson_fd.cc and generated tgmg.cc with oracle/ref_tgmg_driver.cc),
and for each case runs poisson_fd's Gaussian source, the reference's
tgmg<poisson_fd,double,double>::solve_v_cycle(tgmg_predict&) from z = 0 and
records the hierarchy sizes, every coarse level's Galerkin stencils
(tgmg_level::s), the converged z, the V-cycle count and the l2_error after
each of the first V-cycles from zero.  Stored as tests/golden/tgmg_*.npz.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.bind_tgmg import ReferenceTgmg  # noqa: E402

# name -> (m, n, ax, bx, ay, by, Gaussian centre gx, gy, radius, amplitude, keep stencils)
CASES = {
    "tgmg_pfd33": (33, 33, -8.0, 8.0, -8.0, 8.0, 0.0, 0.0, 1.0, 1.0, True),
    "tgmg_pfd65x49": (65, 49, -8.0, 8.0, -6.0, 6.0, 1.5, -0.5, 1.0, 1.0, True),
    "tgmg_pfd40x30": (40, 30, -4.0, 4.0, -3.0, 3.0, -1.0, 0.5, 0.8, 2.0, True),
    "tgmg_pfd17x24": (17, 24, -2.0, 2.0, -3.0, 3.0, 0.2, 0.1, 0.7, 1.0, True),
    "tgmg_pfd129": (129, 129, -8.0, 8.0, -8.0, 8.0, 6.0, 0.0, 1.0, 1.0, False),
}


def make(name, case):
    m, n, ax, bx, ay, by, gx, gy, r, amp, keep = case
    ref = ReferenceTgmg(m, n, ax, bx, ay, by)
    ref.gaussian_source_term(gx, gy, r, amp)
    b = ref.b()
    levels = ref.levels()
    out = {"b": b}
    if keep:
        for l in range(1, len(levels)):
            out["stencil%d" % l] = ref.stencil(l)
    # contraction from zero: l2_error after each of 6 V-cycles
    hist = []
    for _ in range(6):
        ref.v_cycles(1)
        hist.append(ref.l2_error())
    ref.set_z(np.zeros((n, m)))
    ok, iters, lim = ref.solve(4)
    out["z"] = ref.z()
    meta = {"m": m, "n": n, "ax": ax, "bx": bx, "ay": ay, "by": by, "source": [gx, gy, r, amp],
            "levels": levels, "acc": ref.acc, "converged": ok, "vcycles": iters, "lim": lim,
            "l2_after": ref.l2_error(), "l2_history_from_zero": hist}
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    ref.close()
    print(name, "levels", levels, "vcycles", iters, "l2", meta["l2_after"])


def main(argv):
    names = argv[1:] or list(CASES)
    for name in names:
        make(name, CASES[name])


if __name__ == "__main__":
    main(sys.argv)
