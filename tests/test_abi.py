"""CPU-side checks of the C ABI: the library loads, exports every symbol the
header declares, and fails cleanly (status code, no exit) without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from stz_gb300 import _lib
from stz_gb300.params import simple_shear

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols(header="stzg.h"):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(stzg_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from stz_gb300 import build
    build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    names = header_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(_lib.EXPORTS) == names


def test_exports_every_general_multigrid_symbol(lib):
    from stz_gb300 import tgmg
    names = header_symbols("stzg_tgmg.h")
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(tgmg.EXPORTS) == names
    tgmg.load()


def test_exports_every_sheared_step_symbol(lib):
    from stz_gb300 import ct_sim
    names = header_symbols("stzg_ct.h")
    assert len(names) >= 8
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(ct_sim.EXPORTS) == names
    ct_sim.load()


def test_general_multigrid_without_gpu_returns_status(lib):
    import ctypes
    from stz_gb300 import tgmg
    tgmg.load()
    P = ctypes.POINTER(ctypes.c_double)
    IP = ctypes.POINTER(ctypes.c_int)
    table = np.zeros(18)
    cls = np.zeros(9 * 7, dtype=np.int32)
    acc = ctypes.c_double()
    assert lib.stzg_poisson_fd(9, 7, -1.0, 1.0, -1.0, 1.0, table.ctypes.data_as(P), cls.ctypes.data_as(IP),
                               ctypes.byref(acc)) == 0
    from oracle import tgmg_oracle
    t2, c2, a2 = tgmg_oracle.poisson_fd(9, 7, -1.0, 1.0, -1.0, 1.0)
    assert np.array_equal(table.reshape(2, 9), t2) and np.array_equal(cls.reshape(7, 9), c2) and acc.value == a2
    tp = tgmg.Predict()
    assert (tp.lim, tp.mult, tp.decay, tp.max_thresh, tp.extra_iters) == (128, 16, 32, 16 * 2048, 1)
    h = ctypes.c_void_p()
    st = lib.stzg_tgmg_create(9, 7, 0, 0, table.ctypes.data_as(P), 2, cls.ctypes.data_as(IP), acc.value, 0,
                              ctypes.byref(h))
    if not _has_gpu():
        assert st == 7 and not h.value
    else:
        assert st == 0
        lib.stzg_tgmg_destroy(h)


def test_status_strings(lib):
    for code in range(8):
        assert lib.stzg_strerror(code).decode() == _lib.STATUS[code]


def test_create_without_gpu_or_with_bad_args_returns_status(lib):
    h = ctypes.c_void_p()
    bad = simple_shear(15)  # odd m is rejected before touching the device
    st = lib.stzg_create(ctypes.byref(bad), None, ctypes.byref(h))
    assert st == 1 and not h.value
    assert "even" in lib.stzg_last_message().decode()
    P = simple_shear(16)
    st = lib.stzg_create(ctypes.byref(P), None, ctypes.byref(h))
    if not _has_gpu():
        assert st == 7  # no device: status, not an exit
    else:
        assert st == 0
        lib.stzg_destroy(h)


def test_default_options(lib):
    o = _lib.default_options()
    assert o.precision == 0 and o.tol == 1e4 and o.tol_mode == 0 and o.use_graphs == 1


def test_random_chi_matches_oracle(lib):
    from oracle.bind import random_chi as oracle_chi
    from stz_gb300.shear_sim import random_chi
    a = random_chi(48, 40, 4.0, 600.0, 30.0, 21000.0, 5)
    b = oracle_chi(48, 40, 4.0, 600.0, 30.0, 21000.0, 5)
    assert np.max(np.abs(a - b)) <= 1e-15 * np.max(np.abs(b))
    # statistics of the seeded field: mean 600 K, std close to 30 K
    t = a * 21000.0
    assert abs(t.mean() - 600) < 10
    assert 5 < t.std() < 60


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_c_field_pack_unpack_round_trip(lib):
    """The reference's c_field array (19 doubles per point, rows -1..n) to the
    upload buffers and back: cell fields from every row, node fields (X, Y and
    u, v into vel pairs) from rows 0..n, other members untouched."""
    from stz_gb300.shear_sim import C_FIELD_DOUBLES, c_field_pack, c_field_unpack
    m, n = 7, 5
    rng = np.random.default_rng(3)
    rec = rng.standard_normal((n + 2) * m * C_FIELD_DOUBLES).reshape((n + 2) * m, C_FIELD_DOUBLES)
    cells = [np.zeros((n + 2) * m) for _ in range(5)]
    nodes = [np.zeros((n + 1) * m) for _ in range(2)]
    vel = np.zeros(2 * (n + 1) * m)
    soa = cells + nodes + [vel]
    c_field_pack(rec, m, n, soa)
    for q, col in enumerate((2, 3, 4, 5, 6)):
        assert np.array_equal(cells[q], rec[:, col])
    assert np.array_equal(nodes[0], rec[m:, 7]) and np.array_equal(nodes[1], rec[m:, 8])
    assert np.array_equal(vel[0::2], rec[m:, 0]) and np.array_equal(vel[1::2], rec[m:, 1])
    back = rng.standard_normal(rec.shape)
    keep = back.copy()
    c_field_unpack(soa, m, n, back)
    for col in (2, 3, 4, 5, 6):
        assert np.array_equal(back[:, col], rec[:, col])
    for col in (0, 1, 7, 8):
        assert np.array_equal(back[m:, col], rec[m:, col])
        assert np.array_equal(back[:m, col], keep[:m, col])  # row -1 has no node values
    assert np.array_equal(back[:, 9:], keep[:, 9:])
