"""CPU checks of the general-multigrid oracle (oracle/tgmg_oracle.py) against
the golden fixtures the reference's tgmg<poisson_fd,double,double> produced,
and, where the reference tree is present, against the reference build live."""
import numpy as np
import pytest

from oracle import tgmg_oracle as O


def _problem(meta):
    return O.poisson_fd(meta["m"], meta["n"], meta["ax"], meta["bx"], meta["ay"], meta["by"])


def test_poisson_fd_constants_and_source(golden_tgmg):
    name, meta, arr = golden_tgmg
    table, cls, acc = _problem(meta)
    assert acc == meta["acc"]
    gx, gy, r, amp = meta["source"]
    b = O.gaussian_source(meta["m"], meta["n"], meta["ax"], meta["bx"], meta["ay"], meta["by"], gx, gy, r, amp)
    assert np.abs(b - arr["b"]).max() <= 4e-16 * np.abs(arr["b"]).max()


def test_hierarchy_and_galerkin_stencils(golden_tgmg):
    """Level sizes and every coarse stencil equal the reference's rat()."""
    name, meta, arr = golden_tgmg
    table, cls, acc = _problem(meta)
    ops, sizes = O.hierarchy(meta["m"], meta["n"], 0, 0, table, cls)
    assert [list(s) for s in sizes] == meta["levels"]
    for l in range(1, len(sizes)):
        key = "stencil%d" % l
        if key not in arr:
            continue
        cm, cn = sizes[l]
        mine = O.stencils(ops[l], cm, cn, 0, 0)
        ref = arr[key]
        scale = np.abs(ref[..., :9]).max()
        assert np.abs(mine[..., :9] - ref[..., :9]).max() <= 1e-15 * scale, (name, l)
        assert np.allclose(mine[..., 9], ref[..., 9], rtol=1e-14, atol=0)


def test_reference_solution_is_the_discrete_solution(golden_tgmg):
    """The reference's converged z agrees with the exact discrete solution."""
    name, meta, arr = golden_tgmg
    table, cls, acc = _problem(meta)
    A = O.operator(meta["m"], meta["n"], 0, 0, table, cls)
    zx = O.solve(A, arr["b"])
    assert meta["converged"] and meta["l2_after"] < meta["acc"]
    assert np.abs(arr["z"] - zx).max() <= 1e-10 * np.abs(zx).max()
    # near the rounding floor the residual depends on the summation order
    assert O.l2_error(A, arr["z"], arr["b"]) == pytest.approx(meta["l2_after"], rel=1e-3, abs=1e-30)


def test_interpolation_rows_sum_to_one():
    for um in (4, 5, 16, 17):
        for prd in (0, 1):
            P = O.interp_1d(um, prd).toarray()
            assert np.allclose(P.sum(axis=1), 1.0)
            assert P.shape[1] == (um + (1 if prd else 2)) >> 1


def test_live_reference_matches_oracle():
    bt = pytest.importorskip("oracle.bind_tgmg")
    if not bt.available():
        pytest.skip("reference tree not present")
    for (m, n) in ((21, 19), (36, 27)):
        ref = bt.ReferenceTgmg(m, n, -3.0, 3.0, -2.0, 2.0)
        table, cls, acc = O.poisson_fd(m, n, -3.0, 3.0, -2.0, 2.0)
        ops, sizes = O.hierarchy(m, n, 0, 0, table, cls)
        assert ref.levels() == sizes
        for l in range(1, len(sizes)):
            mine = O.stencils(ops[l], sizes[l][0], sizes[l][1], 0, 0)
            ref_s = ref.stencil(l)
            assert np.abs(mine[..., :9] - ref_s[..., :9]).max() <= 1e-15 * np.abs(ref_s[..., :9]).max()
        ref.close()


def _gauss_jordan_pivots(A):
    """Pivots of Gauss-Jordan elimination with partial pivoting (the order
    the GPU solver's dense coarsest inverse uses), relative to max |A|."""
    M = np.array(A, dtype=np.float64)
    amax = np.abs(M).max()
    piv = []
    for c in range(M.shape[0]):
        p = c + int(np.argmax(np.abs(M[c:, c])))
        piv.append(abs(M[p, c]) / amax)
        if p != c:
            M[[p, c]] = M[[c, p]]
        M[c] /= M[c, c]
        col = M[:, c].copy()
        col[c] = 0
        M -= np.outer(col, M[c])
    return np.sort(piv)


def test_singular_coarsest_level_pivots():
    """The coarsest level of a periodic 2x2-block operator that annihilates
    rigid translations (the sheared-coordinates operator with y periodic,
    512x256, seven levels) is singular, but its Galerkin rounding leaves
    pivots between 1e-12 and 1e-8 of its largest entry, with the next pivot
    far above: the solver takes a level as singular below 1e-8, not 1e-12."""
    m, n = 512, 256
    K, mu, lt = 2.5, 1.0, 0.02
    L = K - 2. / 3. * mu
    regh = np.array([[L + 2 * mu + lt * lt * mu, lt * mu + lt ** 3 * mu], [-lt * (L + mu), mu * (1 + lt * lt)]])
    regv = np.array([[mu, lt * mu], [0, L + 2 * mu]])
    regd = np.array([[-0.5 * lt * mu, 0.25 * (L + mu - 2 * lt * lt * mu)], [0.25 * (L + mu), -0.25 * lt * (L + 3 * mu)]])
    ci = np.linalg.inv(-2 * (regh + regv))
    regh, regv, regd = ci @ regh, ci @ regv, ci @ regd
    table = np.stack([regd, regv, -regd, regh, np.eye(2), regh, -regd, regv, regd])[None]
    cls = np.zeros((n, m), dtype=np.int32)
    sizes = O.level_sizes(m, n, 1, 1)
    A = O.operator(m, n, 1, 1, table, cls, 2)
    for l in range(1, len(sizes)):
        A, _ = O.galerkin(A, sizes[l - 1][0], sizes[l - 1][1], 1, 1, 2)
    assert sizes[-1] == (8, 4)
    piv = _gauss_jordan_pivots(A.toarray())
    assert 1e-12 < piv[0] <= piv[1] < 1e-8, piv[:3]
    assert piv[2] > 0.1, piv[:3]
