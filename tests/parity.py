"""Group-normalised parity metric shared by the tests.

Per-field relative error is ill-defined here: under simple shear v, p and q
sit at ~1e-17 by symmetry.  Errors are therefore normalised per field group
(the reference's own comparison, shear_sim::l2_comparison at
esim/sb/main/shear_sim.cc:460-502, groups the fields the same way):
  * stress (p, q, s, tau): max over cells of |p| + sqrt(3q^2+s^2+tau^2);
  * velocity (u, v): the wall speed scale max|u|;
  * chi: max chi;  reference map (X, Y): the domain length;
  * plastic strain eps_pl: its max (or 1e-300 when it is zero everywhere).
"""
import numpy as np

GROUPS = {
    "stress": ("p", "q", "s", "tau"),
    "velocity": ("u", "v"),
    "chi": ("chi",),
    "refmap": ("X", "Y"),
    "eps_pl": ("eps_pl",),
}


def interior(name, a, n):
    """Strip ghost rows of cell fields: (n+2, m) -> (n, m)."""
    if name in ("p", "q", "s", "tau", "chi", "ddev") and a.shape[0] == n + 2:
        return a[1:-1]
    return a


def group_scales(f, n, domain_length=2.0):
    p, q, s, t = (interior(k, f[k], n) for k in ("p", "q", "s", "tau"))
    stress = float(np.max(np.abs(p) + np.sqrt(3 * q * q + s * s + t * t)))
    return {
        "stress": max(stress, 1e-300),
        "velocity": max(float(np.max(np.abs(f["u"]))), 1e-300),
        "chi": float(np.max(np.abs(interior("chi", f["chi"], n)))),
        "refmap": domain_length,
        "eps_pl": max(float(np.max(np.abs(f["eps_pl"]))), 1e-300),
    }


def group_errors(ref, got, n, fields=None):
    """max |got-ref| / scale per group, with ref's scales."""
    sc = group_scales(ref, n)
    out = {}
    for g, names in GROUPS.items():
        e = 0.0
        for k in names:
            if fields is not None and k not in fields:
                continue
            if k not in ref or k not in got:
                continue
            a = interior(k, np.asarray(ref[k]), n)
            b = interior(k, np.asarray(got[k]), n)
            e = max(e, float(np.max(np.abs(a - b))))
        out[g] = e / sc[g]
    return out
