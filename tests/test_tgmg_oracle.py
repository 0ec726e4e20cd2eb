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


def _periodic_block_operator(m, n, lt):
    """The sheared-coordinates operator with x and y periodic (qs_multi.cc
    preconditioned by the inverse centre): singular, rigid translations."""
    K, mu = 2.5, 1.0
    L = K - 2. / 3. * mu
    regh = np.array([[L + 2 * mu + lt * lt * mu, lt * mu + lt ** 3 * mu], [-lt * (L + mu), mu * (1 + lt * lt)]])
    regv = np.array([[mu, lt * mu], [0, L + 2 * mu]])
    regd = np.array([[-0.5 * lt * mu, 0.25 * (L + mu - 2 * lt * lt * mu)], [0.25 * (L + mu), -0.25 * lt * (L + 3 * mu)]])
    ci = np.linalg.inv(-2 * (regh + regv))
    regh, regv, regd = ci @ regh, ci @ regv, ci @ regd
    table = np.stack([regd, regv, -regd, regh, np.eye(2), regh, -regd, regv, regd])[None]
    return table, np.zeros((n, m), dtype=np.int32)


def _emulated_levels(m, n, table, cls, T):
    """Per level: operator, block-diagonal inverse centre and the four colour
    masks of the GPU's Gauss-Seidel, and the interpolation, in type T."""
    import scipy.sparse as sp
    ops, sizes = O.hierarchy(m, n, 1, 1, table, cls, 2)
    lv = []
    for l, ((lm, ln), A) in enumerate(zip(sizes, ops)):
        A = A.tocsr()
        npt = lm * ln
        idx = 2 * np.arange(npt)
        blocks = np.stack([np.stack([np.asarray(A[idx + r, idx + c]).ravel() for c in range(2)], -1)
                           for r in range(2)], 1)
        inv = np.linalg.inv(blocks)
        pi = np.repeat(np.arange(npt), 4)
        Dinv = sp.csr_matrix((inv.reshape(-1), (2 * pi + np.tile([0, 0, 1, 1], npt),
                                                2 * pi + np.tile([0, 1, 0, 1], npt))), shape=(2 * npt, 2 * npt))
        jj, ii = np.divmod(np.arange(npt), lm)
        colors = [np.repeat(((ii & 1) == cx) & ((jj & 1) == cy), 2) for cy in (0, 1) for cx in (0, 1)]
        P = None
        if l + 1 < len(sizes):
            P = sp.kron(sp.kron(O.interp_1d(ln, 1), O.interp_1d(lm, 1)), sp.identity(2), format="csr").astype(T)
        lv.append(dict(A=A.astype(T), A64=A, Dinv=Dinv.astype(T), colors=colors, P=P))
    return lv


def _emulated_vcycle(lv, i, b, T, bottom_inv=None, hb=10):
    """The GPU's V-cycle (one four-colour Gauss-Seidel sweep down and up, the
    coarsest level smoothed 2 hb times or multiplied by bottom_inv), from z = 0."""
    L = lv[i]

    def sweep(z):
        for cm in L["colors"]:
            z = z + np.where(cm, L["Dinv"] @ (b - L["A"] @ z), 0).astype(T)
        return z

    z = np.zeros_like(b)
    if i == len(lv) - 1:
        if bottom_inv is not None:
            return (bottom_inv @ b).astype(T)
        for _ in range(2 * hb):
            z = sweep(z)
        return z
    z = sweep(z)
    zc = _emulated_vcycle(lv, i + 1, (L["P"].T @ (b - L["A"] @ z)).astype(T), T, bottom_inv, hb)
    return sweep((z + L["P"] @ zc).astype(T))


@pytest.mark.parametrize("dense_bottom", [False, True])
def test_mixed_refinement_needs_a_smoothed_singular_bottom(dense_bottom):
    """The mixed-precision solve of the general multigrid, emulated on the CPU
    (FP32 V-cycles of the GPU's ordering on the FP64 residual, corrections
    added in FP64), on the singular periodic operator at 512x256: with the
    coarsest level smoothed it contracts the residual as fast as FP64
    V-cycles; with the dense "inverse" that a 1e-12 pivot test let through
    (entries ~1e10), rounded to FP32, it does not converge."""
    m, n = 512, 256
    table, cls = _periodic_block_operator(m, n, 0.02)
    lv = _emulated_levels(m, n, table, cls, np.float32)
    inv = None
    if dense_bottom:
        inv = np.linalg.inv(lv[-1]["A64"].toarray()).astype(np.float32)
    b = np.random.default_rng(1).standard_normal((n, m, 2)) * 1e-5
    b = (b - b.mean(axis=(0, 1))).ravel()
    A64 = lv[0]["A64"]
    x = np.zeros_like(b)
    l2 = [np.mean(b * b)]
    for _ in range(8):
        r = b - A64 @ x
        x = x + _emulated_vcycle(lv, 0, r.astype(np.float32), np.float32, inv).astype(np.float64)
        r = b - A64 @ x
        l2.append(np.mean(r * r))
    if dense_bottom:
        assert l2[-1] > 1e-3 * l2[0], l2
    else:
        # FP64 V-cycles on this operator: ~0.1 per cycle in the squared residual
        assert l2[-1] < 1e-7 * l2[0], l2
