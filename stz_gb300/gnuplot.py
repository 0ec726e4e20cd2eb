"""Reader and writer of the Gnuplot binary matrix files that the reference
writes for every output frame (shear_sim::output, esim/sb/main/shear_sim.cc:
684-720) and that stzg_write_frame reproduces byte for byte.

Layout, all float32: a first row [L, x_0, ..., x_{L-1}], then one row per
grid line [y_j, f(x_0, y_j), ..., f(x_{L-1}, y_j)].
"""
import numpy as np


def read_matrix(path_or_bytes):
    """Returns (x, y, values) with values of shape (len(y), len(x))."""
    if isinstance(path_or_bytes, (bytes, bytearray)):
        a = np.frombuffer(path_or_bytes, dtype=np.float32)
    else:
        a = np.fromfile(path_or_bytes, dtype=np.float32)
    width = int(a[0]) + 1
    if width < 2 or a.size % width:
        raise ValueError("not a Gnuplot binary matrix")
    m = a.reshape(-1, width)
    return m[0, 1:].copy(), m[1:, 0].copy(), m[1:, 1:].copy()


def write_matrix(path, x, y, values):
    """Writes the same layout from coordinates and a (len(y), len(x)) array."""
    x = np.asarray(x, dtype=np.float32)
    y = np.asarray(y, dtype=np.float32)
    v = np.asarray(values, dtype=np.float32).reshape(len(y), len(x))
    out = np.empty((len(y) + 1, len(x) + 1), dtype=np.float32)
    out[0, 0] = len(x)
    out[0, 1:] = x
    out[1:, 0] = y
    out[1:, 1:] = v
    out.tofile(path)
