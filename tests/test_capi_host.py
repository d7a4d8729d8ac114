"""Host-side checks of the C ABI that need no GPU: the library loads and
exports every entry point include/rpp_gb300.h declares, the native Hall basis
and conversion matrices equal the reference's (golden fixtures), argument
validation reports the reference's error codes, and the division-by-width
arithmetic used by the kernels is exact."""
import ctypes
import importlib
import os
import re

import numpy as np
import pytest

pkg = importlib.import_module("rough-path-primitives_gb300")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            with open(os.path.join(ROOT, "include", fn)) as f:
                text = f.read()
            names |= set(re.findall(r"^\s*(?:int|const char\*)\s+(rpp_gb_\w+)\s*\(", text, re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = pkg.library()
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(pkg._lib.SIGNATURES) >= names
    assert lib.rpp_gb_version().decode().startswith("rpp_gb300")


@pytest.mark.parametrize("wd", [(3, 4), (4, 4), (5, 5), (2, 6)])
def test_native_lie_tables_match_reference(golden_dir, wd):
    z = np.load(os.path.join(golden_dir, f"lie_{wd[0]}_{wd[1]}.npz"))
    lb = pkg.LieBasis(*wd)
    assert lb.degree_begin == z["degree_begin"].tolist()
    assert np.array_equal(lb.pairs, z["pairs"])
    for name, m in (("t2l", pkg.make_t2l_matrix(lb)), ("l2t", pkg.make_l2t_matrix(lb))):
        assert np.array_equal(m.offsets, z[f"{name}_offsets"])
        assert np.array_equal(m.indices, z[f"{name}_indices"])
        assert np.array_equal(m.values, z[f"{name}_values"])
        assert (m.outer_dim, m.inner_dim) == tuple(z[f"{name}_dims"].tolist())


def test_native_lie_tables_match_oracle_large():
    """W6 D6 (9695 Lie elements): native builder vs the Python oracle's."""
    import oracle as O

    tab = O.LieTables(4, 6)
    lb = pkg.LieBasis(4, 6)
    assert lb.degree_begin == tab.db
    m = pkg.make_t2l_matrix(lb)
    off, idx, val, dims = tab.t2l_csc()
    assert np.array_equal(m.offsets, off) and np.array_equal(m.indices, idx) and np.array_equal(m.values, val)


def test_errors_without_a_device():
    lib = pkg.library()
    t = pkg._lib.TensorArg(0, 0, 0, 0)
    rc = lib.rpp_gb_ft_mul(None, None, 1, ctypes.byref(t), ctypes.byref(t), ctypes.byref(t), 1, 1.0)
    assert rc == int(pkg.ErrorCode.InvalidArgument)
    assert b"plan" in lib.rpp_gb_last_error_string()
    out = ctypes.c_void_p()
    assert lib.rpp_gb_plan_create(ctypes.byref(out), 0, 3, 0) == int(pkg.ErrorCode.InvalidArgument)
    assert lib.rpp_gb_plan_create(ctypes.byref(out), 3, 31, 0) == int(pkg.ErrorCode.InvalidArgument)
    assert lib.rpp_gb_plan_create(ctypes.byref(out), 255, 5, 0) == int(pkg.ErrorCode.OutOfBounds)
    assert lib.rpp_gb_lie_basis(0, 3, None, None, None) == int(pkg.ErrorCode.InvalidArgument)
    off = np.array([0, 2], np.int64)
    idx = np.array([0, 5], np.int64)
    val = np.array([1.0, 2.0])
    P = ctypes.POINTER(ctypes.c_int64)
    rc = lib.rpp_gb_matrix_create(ctypes.byref(out), 0, 1, 3, 2, off.ctypes.data_as(P), idx.ctypes.data_as(P),
                                  val.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0)
    assert rc == int(pkg.ErrorCode.OutOfBounds)


def fastdiv(d):
    """Host model of FastDiv (csrc/common.cuh): Granlund-Montgomery multiply-high."""
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    return lambda n: (((m * n) >> 32) + n) >> l


@pytest.mark.parametrize("d", [1, 2, 3, 5, 6, 7, 8, 16, 100, 255])
def test_fastdiv_exact(d):
    f = fastdiv(d)
    rng = np.random.default_rng(d)
    ns = list(range(0, 5000)) + rng.integers(0, 2**31, 20000).tolist() + [2**31 - 1, 2**32 - 1]
    for n in ns:
        assert f(n) == n // d, (d, n)
