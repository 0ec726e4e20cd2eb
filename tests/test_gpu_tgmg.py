"""Parity of the general GPU multigrid (include/stzg_tgmg.h) with the
reference's tgmg<poisson_fd,double,double> (golden fixtures) and with the CPU
restatement of its operator algebra (oracle/tgmg_oracle.py): hierarchy sizes,
Galerkin stencils, converged solutions of every solver type, periodic
variants, the predictor's failure path and argument errors."""
import numpy as np
import pytest

from oracle import tgmg_oracle as O

pytestmark = pytest.mark.gpu


def _tg():
    from stz_gb300 import tgmg
    return tgmg


def _pfd(meta):
    tg = _tg()
    q = tg.PoissonFD(meta["m"], meta["n"], meta["ax"], meta["bx"], meta["ay"], meta["by"])
    return q


def test_hierarchy_and_stencils_match_reference(golden_tgmg):
    name, meta, arr = golden_tgmg
    tg = _tg()
    q = _pfd(meta)
    assert q.acc == meta["acc"]
    g = tg.Tgmg(q)
    assert [list(s) for s in g.levels()] == meta["levels"]
    for l in range(1, len(meta["levels"])):
        key = "stencil%d" % l
        if key not in arr:
            continue
        mine, ref = g.stencil(l), arr[key]
        scale = np.abs(ref[..., :9]).max()
        assert np.abs(mine[..., :9] - ref[..., :9]).max() <= 1e-15 * scale, (name, l)
    g.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_vcycle_solve_matches_reference(golden_tgmg, mixed):
    """solve_v_cycle(tgmg_predict&) from z = 0 on the reference's source:
    converged under acc, and the solution agrees with the reference's and with
    the exact discrete solution; in mixed precision (FP32 V-cycles inside FP64
    refinement) with as many passes as the reference's V-cycles."""
    name, meta, arr = golden_tgmg
    tg = _tg()
    q = _pfd(meta)
    q.b[...] = arr["b"]
    g = tg.Tgmg(q)
    if mixed:
        g.set_precision(True)
    tp = tg.Predict()
    assert g.solve_v_cycle(tp)
    assert g.l2_error() < q.acc
    table, cls, acc = O.poisson_fd(meta["m"], meta["n"], meta["ax"], meta["bx"], meta["ay"], meta["by"])
    zx = O.solve(O.operator(meta["m"], meta["n"], 0, 0, table, cls), arr["b"])
    scale = np.abs(zx).max()
    assert np.abs(q.z - zx).max() <= 1e-9 * scale
    assert np.abs(q.z - arr["z"]).max() <= 1e-9 * scale
    # the GPU's four-colour V-cycle needs about as many cycles as the
    # reference's zebra ordering
    assert g.iterations <= meta["vcycles"] + 2
    g.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_checked_solve(golden_tgmg, mixed):
    """stzg_tgmg_solve_checked: from z = 0 it converges with no more V-cycles
    (passes) than the reference needed plus two and agrees with the
    reference's solution; from a converged z it runs none but the extra one."""
    name, meta, arr = golden_tgmg
    tg = _tg()
    q = _pfd(meta)
    q.b[...] = arr["b"]
    g = tg.Tgmg(q)
    g.set_precision(mixed)
    assert g.solve_v_cycle_checked()
    assert g.iterations <= meta["vcycles"] + 2
    assert g.residual < q.acc and g.l2_error() < q.acc
    scale = np.abs(arr["z"]).max()
    assert np.abs(q.z - arr["z"]).max() <= 1e-9 * scale
    assert g.solve_v_cycle_checked()
    assert g.iterations == 0
    g.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_vcycle_contraction_from_zero(golden_tgmg, mixed):
    name, meta, arr = golden_tgmg
    tg = _tg()
    q = _pfd(meta)
    q.b[...] = arr["b"]
    g = tg.Tgmg(q)
    if mixed:
        g.set_precision(True)
    hist = []
    for _ in range(6):
        g.v_cycle()
        hist.append(g.l2_error())
    ref = meta["l2_history_from_zero"]
    # l2_error is squared: the reference contracts it by 0.003-0.015 a cycle
    for k in range(1, 4):
        assert hist[k] <= 0.05 * hist[k - 1] or hist[k] < q.acc
        assert hist[k] <= 10 * ref[k] or hist[k] < q.acc
    g.close()


@pytest.mark.parametrize("kind", ["fmg", "sym", "fixed_v", "fixed_fmg"])
def test_other_multigrid_solvers(kind):
    tg = _tg()
    q = tg.PoissonFD(40, 30, -4.0, 4.0, -3.0, 3.0)
    q.gaussian_source_term(0.3, -0.2, 0.8, 1.0)
    b = q.b.copy()
    g = tg.Tgmg(q)
    tp = tg.Predict()
    ok = {"fmg": lambda: g.solve_full_multigrid(tp), "sym": lambda: g.solve_sym_v_cycle(tp),
          "fixed_v": lambda: g.solve_v_cycle(), "fixed_fmg": lambda: g.solve_full_multigrid()}[kind]()
    assert ok and g.l2_error() < q.acc
    zx = O.solve(O.operator(40, 30, 0, 0, q.table, q.cls), b)
    assert np.abs(q.z - zx).max() <= 1e-9 * np.abs(zx).max()
    g.close()


@pytest.mark.parametrize("kind", ["jacobi", "gs", "sor"])
def test_relaxation_solvers(kind):
    tg = _tg()
    q = tg.PoissonFD(9, 8, -1.0, 1.0, -1.0, 1.0)
    q.gaussian_source_term(0.0, 0.0, 0.5, 1.0)
    b = q.b.copy()
    g = tg.Tgmg(q)
    ok = {"jacobi": lambda: g.solve_jacobi(), "gs": lambda: g.solve_gauss_seidel(),
          "sor": lambda: g.solve_sor(1.5)}[kind]()
    assert ok and g.l2_error() <= q.acc
    zx = O.solve(O.operator(9, 8, 0, 0, q.table, q.cls), b)
    assert np.abs(q.z - zx).max() <= 1e-8 * np.abs(zx).max()
    g.close()


def _helmholtz(m, n, xp, yp, rows_vary=False, seed=0):
    """A 9-point operator with a shifted diagonal (nonsingular on periodic
    grids), optionally with per-row coefficients and corner entries."""
    rng = np.random.default_rng(seed)
    if rows_vary:
        table = []
        for j in range(n):
            a = 1.0 + 0.5 * rng.random()
            c = 0.1 * rng.random()
            table.append([c, a, c, 1.0, -(2 * a + 2 + 4 * c) - 0.3, 1.0, c, a, c])
        table = np.array(table)
        cls = np.repeat(np.arange(n, dtype=np.int32)[:, None], m, axis=1)
    else:
        table = np.array([[0, 1.0, 0, 1.0, -4.3, 1.0, 0, 1.0, 0]])
        cls = np.zeros((n, m), dtype=np.int32)
    return table, cls


@pytest.mark.parametrize("m,n,xp,yp,vary", [(32, 24, 1, 0, False), (33, 25, 1, 0, False), (24, 32, 0, 1, False),
                                            (27, 21, 1, 1, False), (40, 36, 1, 1, True), (31, 17, 0, 0, True)])
def test_periodic_and_variable_operators(m, n, xp, yp, vary):
    tg = _tg()
    table, cls = _helmholtz(m, n, xp, yp, vary, seed=m * n)
    ops, sizes = O.hierarchy(m, n, xp, yp, table, cls)
    q = tg.Problem(m, n, table, cls, 1e-26, x_prd=xp, y_prd=yp)
    rng = np.random.default_rng(1)
    q.b[...] = rng.standard_normal((n, m))
    b = q.b.copy()
    g = tg.Tgmg(q)
    assert g.levels() == sizes
    for l in range(1, len(sizes)):
        mine = g.stencil(l)
        ref = O.stencils(ops[l], sizes[l][0], sizes[l][1], xp, yp)
        assert np.abs(mine[..., :9] - ref[..., :9]).max() <= 1e-14 * np.abs(ref[..., :9]).max(), l
    tp = tg.Predict()
    assert g.solve_v_cycle(tp)
    zx = O.solve(ops[0], b)
    assert np.abs(q.z - zx).max() <= 1e-10 * np.abs(zx).max()
    g.close()


def test_predictor_threshold_returns_false():
    """The reference returns false once lim exceeds max_thresh; so does the
    mirror, with a status and no fault."""
    tg = _tg()
    q = tg.PoissonFD(33, 33, -8.0, 8.0, -8.0, 8.0)
    q.gaussian_source_term(0, 0, 1, 1)
    q.acc = 0.0  # unreachable
    g = tg.Tgmg(q)
    tp = tg.Predict()
    tp.max_thresh = tp.lim + 3 * tp.mult
    assert g.solve_v_cycle(tp) is False
    g.close()


def test_bad_arguments_are_statuses():
    import ctypes
    tg = _tg()
    lib = tg.load()
    h = ctypes.c_void_p()
    table = np.array([0, 1, 0, 1, -4, 1, 0, 1, 0], dtype=np.float64)
    cls = np.zeros(4, dtype=np.int32)
    P = ctypes.POINTER(ctypes.c_double)
    IP = ctypes.POINTER(ctypes.c_int)
    # periodic line of 2 points
    assert lib.stzg_tgmg_create(2, 2, 1, 0, table.ctypes.data_as(P), 1, cls.ctypes.data_as(IP), 0.0, 0,
                                ctypes.byref(h)) == 1
    cls[1] = 3  # index out of range
    assert lib.stzg_tgmg_create(2, 2, 0, 0, table.ctypes.data_as(P), 1, cls.ctypes.data_as(IP), 0.0, 0,
                                ctypes.byref(h)) == 1
    assert not h.value
    # a valid solver: bad precision, bad checked-solve limits, a kept class
    # map with another stencil count
    cls[1] = 0
    assert lib.stzg_tgmg_create(2, 2, 0, 0, table.ctypes.data_as(P), 1, cls.ctypes.data_as(IP), 0.0, 0,
                                ctypes.byref(h)) == 0
    assert lib.stzg_tgmg_set_precision(h, 2) == 1
    it, l2 = ctypes.c_int(), ctypes.c_double()
    assert lib.stzg_tgmg_solve_checked(h, 4, -1, 1, ctypes.c_double(1.0), 1, 1, 10, ctypes.byref(it),
                                       ctypes.byref(l2)) == 1
    two = np.concatenate([table, table])
    assert lib.stzg_tgmg_set_operator(h, two.ctypes.data_as(P), 2, None) == 1
    assert lib.stzg_tgmg_destroy(h) == 0


def test_reports_device_time_and_kernels():
    tg = _tg()
    q = tg.PoissonFD(129, 129, -8.0, 8.0, -8.0, 8.0)
    q.gaussian_source_term(1, 1, 1, 1)
    g = tg.Tgmg(q)
    g.v_cycle()
    ms, k = g.last_timing()
    assert ms > 0 and k > 10
    g.close()


def test_cpp_dropin_header(tmp_path):
    """include/stzg_tgmg.hh with a problem class of the reference's concept,
    compiled into a small driver, reproduces the reference's solution."""
    import json
    import os
    import subprocess
    from conftest import GOLDEN
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = os.path.join(root, "stz_gb300", "_build")
    exe = tmp_path / "tgmg_main"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(root, "include"),
                           os.path.join(root, "tests", "cpp", "tgmg_main.cc"), "-o", str(exe), "-L", lib, "-lstzg",
                           f"-Wl,-rpath,{lib}"])
    d = np.load(os.path.join(GOLDEN, "tgmg_pfd65x49.npz"))
    meta = json.loads(str(d["meta"]))
    bfile, zfile = tmp_path / "b.bin", tmp_path / "z.bin"
    d["b"].astype(np.float64).tofile(bfile)
    r = subprocess.run([str(exe), str(meta["m"]), str(meta["n"]), repr(meta["ax"]), repr(meta["bx"]),
                        repr(meta["ay"]), repr(meta["by"]), str(bfile), str(zfile)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    z = np.fromfile(zfile).reshape(meta["n"], meta["m"])
    assert np.abs(z - d["z"]).max() <= 1e-9 * np.abs(d["z"]).max()
    assert "levels %d" % len(meta["levels"]) in r.stdout


def _block_operator(m, n, xp, yp, lt=0.3, seed=0, walls=True):
    """2x2-block operators of the qs_multi kind: horizontal, vertical and
    corner blocks (the transformed operator of coord_transforms qs_multi.cc
    with shear lt, preconditioned by the inverse centre) and, unless y is
    periodic, wall rows that carry only the identity (qs_multi.hh:31-42)."""
    K, mu, h = 2.5, 1.0, 1.0
    L = K - 2. / 3. * mu
    ltsq = lt * lt
    regh = np.array([[(L + 2 * mu + ltsq * mu), (lt * mu + lt * ltsq * mu)], [-lt * (L + mu), mu * (1 + ltsq)]]) / h
    regv = np.array([[mu, lt * mu], [0, (L + 2 * mu)]]) / h
    regc = -2 * (regh + regv)
    regd = np.array([[-0.5 * lt * mu, 0.25 * (L + mu - 2 * ltsq * mu)],
                     [0.25 * (L + mu), -0.25 * lt * (L + 3 * mu)]]) / h
    ci = np.linalg.inv(regc)
    regh, regv, regd = ci @ regh, ci @ regv, ci @ regd
    I2 = np.eye(2)
    inner = np.stack([regd, regv, -regd, regh, I2, regh, -regd, regv, regd])
    wall = np.stack([np.zeros((2, 2))] * 4 + [I2] + [np.zeros((2, 2))] * 4)
    table = np.stack([inner, wall])
    cls = np.zeros((n, m), dtype=np.int32)
    if walls and not yp:
        cls[0, :] = cls[-1, :] = 1
    return table, cls


def test_block_operator_update_class_map():
    """set_operator with a changed class map, and with the map kept (cls
    NULL, only new stencil values): after each update the solver iterates bit
    for bit like one created with that operator (the iteration graph captured
    before an update that moves no table stays valid), and a kept map with
    another stencil count is an error."""
    tg = _tg()
    from stz_gb300 import _lib
    m, n = 40, 24
    t0, cls0 = _block_operator(m, n, 1, 0, lt=0.1)
    t1, _ = _block_operator(m, n, 1, 0, lt=0.45)
    cls1 = cls0.copy()
    cls1[n // 2, :] = 1  # an interior wall row: another stencil pattern
    b = np.random.default_rng(6).standard_normal((n, m, 2))

    def run(g, q):
        q.b[...] = b
        q.z[...] = 0
        for _ in range(3):
            g.v_cycle()
        nl = len(g.levels())
        return [q.z.copy(), g.stencil(1), g.stencil(nl - 1)]

    q = tg.Problem(m, n, t0, cls0, 1e-26, x_prd=True, y_prd=False, block=2)
    g = tg.Tgmg(q)
    run(g, q)
    for t, c, keep in ((t1, cls1, False), (t0, None, True), (t1, None, True), (t1, cls1, False)):
        g.set_operator(t, None if keep else c, keep_classes=keep)
        qf = tg.Problem(m, n, t, cls1, 1e-26, x_prd=True, y_prd=False, block=2)
        gf = tg.Tgmg(qf)
        for x, y in zip(run(g, q), run(gf, qf)):
            assert np.array_equal(x, y)
        gf.close()
    with pytest.raises(_lib.StzgError):
        g.set_operator(np.concatenate([t0, t0[:1]]), keep_classes=True)
    g.close()


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("m,n,xp,yp", [(32, 17, 1, 0), (40, 24, 1, 1), (33, 27, 1, 1), (24, 19, 0, 0)])
def test_block_operators(m, n, xp, yp, mixed):
    """tgmg<S,vec,mat>: Galerkin blocks and the converged solution of
    qs_multi-type 2x2-block operators, periodic or walled in y, in FP64 and
    in mixed precision; a solver switched back to FP64 solves bit for bit
    like one that never left it."""
    tg = _tg()
    table, cls = _block_operator(m, n, xp, yp, seed=m)
    ops, sizes = O.hierarchy(m, n, xp, yp, table, cls, 2)
    q = tg.Problem(m, n, table, cls, 1e-26, x_prd=xp, y_prd=yp, block=2)
    rng = np.random.default_rng(3)
    b = rng.standard_normal((n, m, 2))
    if yp:
        # periodic in both directions the operator annihilates rigid
        # translations: the source must be consistent (zero mean), as the
        # divergence of a stress is
        b -= b.mean(axis=(0, 1))
    q.b[...] = b
    g = tg.Tgmg(q)
    assert g.levels() == sizes
    for l in range(1, len(sizes)):
        mine = g.stencil(l)
        ref = O.stencils(ops[l], sizes[l][0], sizes[l][1], xp, yp, 2)
        assert np.abs(mine[:, :, :9] - ref[:, :, :9]).max() <= 1e-13 * np.abs(ref[:, :, :9]).max(), l
    if mixed:
        g.set_precision(True)
    tp = tg.Predict()
    assert g.solve_v_cycle(tp)
    assert g.l2_error() < q.acc
    if yp:
        zx = np.linalg.lstsq(ops[0].toarray(), b.ravel(), rcond=None)[0].reshape(b.shape)
        got = q.z - q.z.mean(axis=(0, 1))
        zx -= zx.mean(axis=(0, 1))
    else:
        zx, got = O.solve(ops[0], b), q.z
    assert np.abs(got - zx).max() <= 1e-10 * np.abs(zx).max()
    assert g.l2_error() == pytest.approx(O.l2_error(ops[0], q.z, b, 2), rel=1e-3, abs=1e-28)
    if mixed:
        g.set_precision(False)
        q.z[...] = 0
        assert g.solve_v_cycle(tg.Predict())
        q2 = tg.Problem(m, n, table, cls, 1e-26, x_prd=xp, y_prd=yp, block=2)
        q2.b[...] = b
        g2 = tg.Tgmg(q2)
        assert g2.solve_v_cycle(tg.Predict())
        assert np.array_equal(q.z, q2.z)
        g2.close()
    g.close()


@pytest.mark.parametrize("lt", [0.0, 0.02])
def test_block_operator_periodic_large(lt):
    """A singular periodic 2x2-block operator large enough that its coarsest
    level's rounding pivots reach 1e-11..4e-10 of its largest entry (512x256,
    eight levels): the coarsest level is recognised as singular and smoothed,
    and FP64 V-cycles and mixed-precision passes both converge to acc."""
    tg = _tg()
    m, n = 512, 256
    table, cls = _block_operator(m, n, 1, 1, lt=lt)
    b = np.random.default_rng(1).standard_normal((n, m, 2)) * 1e-5
    b -= b.mean(axis=(0, 1))
    its = []
    for mixed in (False, True):
        q = tg.Problem(m, n, table, cls, (2.220446049250313e-16 * 1e4 * 2) ** 2, x_prd=1, y_prd=1, block=2)
        q.b[...] = b
        g = tg.Tgmg(q)
        g.set_precision(mixed)
        assert g.solve_v_cycle_checked(max_iters=40)
        assert g.residual < q.acc
        its.append(g.iterations)
        g.close()
    assert its[1] <= its[0] + 2, its


def test_block_operator_update():
    """set_operator (qs_multi::init + setup on a new shear): the rebuilt
    hierarchy equals a fresh one, and solves keep converging."""
    tg = _tg()
    m, n = 40, 24
    t0, cls = _block_operator(m, n, 1, 0, lt=0.1)
    t1, _ = _block_operator(m, n, 1, 0, lt=0.45)
    q = tg.Problem(m, n, t0, cls, 1e-26, x_prd=True, y_prd=False, block=2)
    q.cls[0, :] = q.cls[-1, :] = 1
    cls = q.cls.copy()
    q.b[...] = np.random.default_rng(5).standard_normal((n, m, 2))
    b = q.b.copy()
    g = tg.Tgmg(q)
    tp = tg.Predict()
    assert g.solve_v_cycle(tp)
    g.set_operator(t1)
    q.z[...] = 0
    assert g.solve_v_cycle(tp)
    ops, sizes = O.hierarchy(m, n, 1, 0, t1, cls, 2)
    zx = O.solve(ops[0], b)
    assert np.abs(q.z - zx).max() <= 1e-10 * np.abs(zx).max()
    ref = O.stencils(ops[1], sizes[1][0], sizes[1][1], 1, 0, 2)
    assert np.abs(g.stencil(1)[:, :, :9] - ref[:, :, :9]).max() <= 1e-13 * np.abs(ref[:, :, :9]).max()
    g.close()
