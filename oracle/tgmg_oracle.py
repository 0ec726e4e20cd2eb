"""CPU restatement of the general tgmg multigrid's operator algebra.

TEST INFRASTRUCTURE ONLY: imported by tests/ and by the golden-fixture
script as the checker of the GPU path (stz_gb300/csrc/tgmg.cu), never by the
product.

Restates, with sparse matrices instead of point loops:
* the problem operator of a tgmg problem class (the stencil functions
  a_dl..a_ur, a_cc of esim/tgmg/poisson_fd.hh:40-56, applied by mul_a with
  neighbours outside a non-periodic grid left out);
* the hierarchy sizes (tgmg_base constructor, tgmg.hh:108-110; levels while
  the child has more than tgmg_grid_min = 10 points, tgmg.in.cc:17-31);
* the one-dimensional interpolation of apply_t / t_line
  (tgmg.in.cc:552-621): even fine points inject, odd ones average their two
  coarse neighbours, the last point of an even non-periodic line injects the
  last coarse point, and an even periodic line wraps;
* the Galerkin products P^T A P of tgmg_base::rat (tgmg.in.cc:667-736) and
  their 9-point stencils in the tgmg_level::s layout (tgmg.hh:235);
* poisson_fd's constants and Gaussian source (poisson_fd.cc:12-39) and the
  l2_error measure mds/mn (tgmg.hh:146, tgmg.in.cc:55-65);
* the exact discrete solution by a sparse direct solve.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

GRID_MIN = 10


def level_sizes(m, n, xp, yp):
    """(m, n) of the top level and every child (periodic lines stop at 3)."""
    out = [(m, n)]
    am, an = (m + (1 if xp else 2)) >> 1, (n + (1 if yp else 2)) >> 1
    while am * an > GRID_MIN and len(out) < 17 and (not xp or am >= 3) and (not yp or an >= 3):
        out.append((am, an))
        am, an = (am + (1 if xp else 2)) >> 1, (an + (1 if yp else 2)) >> 1
    return out


def interp_1d(um, prd):
    """Sparse um x sm interpolation matrix of one direction."""
    sm = (um + (1 if prd else 2)) >> 1
    rows, cols, vals = [], [], []
    for f in range(um):
        if f % 2 == 0:
            ent = [(f >> 1, 1.0)]
        elif not prd and um % 2 == 0 and f == um - 1:
            ent = [(sm - 1, 1.0)]
        else:
            ent = [(f >> 1, 0.5), (0 if (prd and f == um - 1) else (f >> 1) + 1, 0.5)]
        for c, w in ent:
            rows.append(f)
            cols.append(c)
            vals.append(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(um, sm))


def _nbr(i, d, m, prd):
    k = i + d
    if 0 <= k < m:
        return k
    if not prd:
        return -1
    return k + m if k < 0 else k - m


def operator(m, n, xp, yp, table, cls, block=1):
    """Sparse (B m n) x (B m n) operator from a stencil table (dl dc dr cl cc
    cr ul uc ur per row; 2x2 row-major blocks when block = 2) and a stencil
    index per point (index j*m+i); unknown B*(j*m+i)+c."""
    B = block
    table = np.asarray(table, dtype=np.float64).reshape(-1, 9, B, B)
    cls = np.asarray(cls).reshape(-1)
    rows, cols, vals = [], [], []
    ii, jj = np.meshgrid(np.arange(m), np.arange(n))
    ii, jj = ii.ravel(), jj.ravel()
    for sy in (-1, 0, 1):
        ly = np.array([_nbr(j, sy, n, yp) for j in range(n)])[jj]
        for sx in (-1, 0, 1):
            lx = np.array([_nbr(i, sx, m, xp) for i in range(m)])[ii]
            for r in range(B):
                for c in range(B):
                    a = table[cls, (sy + 1) * 3 + sx + 1, r, c]
                    ok = (lx >= 0) & (ly >= 0) & (a != 0)
                    rows.append(B * (jj * m + ii)[ok] + r)
                    cols.append(B * (ly * m + lx)[ok] + c)
                    vals.append(a[ok])
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    return sp.csr_matrix((vals, (rows, cols)), shape=(B * m * n, B * m * n))


def galerkin(A, m, n, xp, yp, block=1):
    """P^T A P and the child size (P acts on every block component)."""
    Px, Py = interp_1d(m, xp), interp_1d(n, yp)
    P = sp.kron(sp.kron(Py, Px), sp.identity(block), format="csr")
    return (P.T @ A @ P).tocsr(), (Px.shape[1], Py.shape[1])


def stencils(A, m, n, xp, yp, block=1):
    """Stencils of a level's operator: (n, m, 10) with the 9 entries and
    1/centre, or (n, m, 10, 2, 2) with the blocks and the inverse centre."""
    B = block
    A = A.tocsr()
    out = np.zeros((n, m, 10, B, B))
    for j in range(n):
        for i in range(m):
            p = j * m + i
            for sy in (-1, 0, 1):
                ly = _nbr(j, sy, n, yp)
                if ly < 0:
                    continue
                for sx in (-1, 0, 1):
                    lx = _nbr(i, sx, m, xp)
                    if lx < 0:
                        continue
                    q = ly * m + lx
                    out[j, i, (sy + 1) * 3 + sx + 1] = A[B * p:B * p + B, B * q:B * q + B].toarray()
            out[j, i, 9] = np.linalg.inv(out[j, i, 4])
    return out[..., 0, 0] if B == 1 else out


def hierarchy(m, n, xp, yp, table, cls, block=1):
    """Operators of every level, top first, and their sizes."""
    sizes = level_sizes(m, n, xp, yp)
    ops = [operator(m, n, xp, yp, table, cls, block)]
    for l in range(1, len(sizes)):
        Ac, csz = galerkin(ops[-1], sizes[l - 1][0], sizes[l - 1][1], xp, yp, block)
        assert csz == sizes[l]
        ops.append(Ac)
    return ops, sizes


def poisson_fd(m, n, ax, bx, ay, by):
    """Stencil table (interior, edge), indices and acc of poisson_fd."""
    dx, dy = (bx - ax) / (m - 1), (by - ay) / (n - 1)
    hcc = -2 / (dx * dx) - 2 / (dy * dy)
    hxx, hyy = 1. / (dx * dx), 1. / (dy * dy)
    a = np.finfo(np.float64).eps * 1e4 * hcc
    table = np.array([[0, hyy, 0, hxx, hcc, hxx, 0, hyy, 0], [0, 0, 0, 0, hcc, 0, 0, 0, 0]], dtype=np.float64)
    cls = np.zeros((n, m), dtype=np.int32)
    cls[0, :] = cls[-1, :] = cls[:, 0] = cls[:, -1] = 1
    return table, cls, a * a


def gaussian_source(m, n, ax, bx, ay, by, gx, gy, r, amp):
    """poisson_fd::gaussian_source_term with x advanced by repeated addition."""
    dx, dy = (bx - ax) / (m - 1), (by - ay) / (n - 1)
    lam = -0.5 / (r * r)
    xs = np.add.accumulate(np.concatenate(([ax - gx], np.full(m - 1, dx))))
    b = np.empty((n, m))
    for j in range(n):
        y = ay - gy + dy * j
        b[j] = amp * np.exp(lam * (xs * xs + y * y))
    return b


def l2_error(A, z, b, block=1):
    """mds/mn: squared residual summed over components, per grid point."""
    r = b.ravel() - A @ z.ravel()
    return float(r @ r) / (r.size // block)


def solve(A, b):
    """Exact discrete solution (b in the unknowns' order, any shape)."""
    return spla.spsolve(A.tocsc(), b.ravel()).reshape(b.shape)
