"""The Gnuplot binary matrix format of the reference's frame files, on the
fixture the reference itself wrote (tests/golden/frames_*.npz)."""
import numpy as np

from stz_gb300.gnuplot import read_matrix, write_matrix


def test_reference_frames_decode(golden_frames, tmp_path):
    name, P, meta, ref = golden_frames
    m, n = P.m, P.n
    # cell field p: n rows of m values at cell centres, the state's rows 0..n-1
    x, y, p = read_matrix(ref["output2"].tobytes())
    assert len(x) == m and len(y) == n
    np.testing.assert_array_equal(p, ref["p"][1:-1].astype(np.float32))
    dx = (P.bx - P.ax) / m
    np.testing.assert_allclose(x, P.ax + (np.arange(m) + 0.5) * dx, rtol=1e-6)
    # node field X: n+1 rows of m+1 values, the last column the periodic copy + lx
    x, y, X = read_matrix(ref["output9"].tobytes())
    assert len(x) == m + 1 and len(y) == n + 1
    np.testing.assert_array_equal(X[:, :m], ref["X"].astype(np.float32))
    np.testing.assert_allclose(X[:, m], X[:, 0] + (P.bx - P.ax), rtol=1e-6)
    # round trip through the writer
    write_matrix(tmp_path / "p.0", *read_matrix(ref["output2"].tobytes()))
    assert (tmp_path / "p.0").read_bytes() == ref["output2"].tobytes()
