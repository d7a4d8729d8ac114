"""The CPU oracle's shuffle-algebra operations reproduce the reference's own
outputs (tests/golden/shuffle_w3d4.npz, written by tests/golden/make_golden.py
from the unmodified reference CPU strategy)."""
import os

import numpy as np
import pytest

from _helpers import assert_close, shuffle_cases

FILE = "shuffle_w3d4.npz"


@pytest.fixture(scope="module")
def sh(golden_dir):
    return np.load(os.path.join(golden_dir, FILE))


def _r(ranges):
    return tuple(tuple(int(v) for v in r) for r in ranges)


def test_st_mul(orc, sh):
    x, y, init = sh["inputs/x"], sh["inputs/y"], sh["inputs/init"]
    for c in shuffle_cases(sh, "st_mul"):
        out = init.copy()
        orc.st_mul(3, 4, out, x, y, _r(c["ranges"]), float(c["beta"]))
        assert_close(out, c["out"], what=f"st_mul {c['ranges'].tolist()}")


def test_st_fma_and_inplace(orc, sh):
    x, y, z, init = sh["inputs/x"], sh["inputs/y"], sh["inputs/z"], sh["inputs/init"]
    for c in shuffle_cases(sh, "st_fma"):
        out = init.copy()
        orc.st_fma(3, 4, out, z, x, y, _r(c["ranges"]), float(c["alpha"]), float(c["beta"]))
        assert_close(out, c["out"], what=f"st_fma {c['ranges'].tolist()}")
    for c in shuffle_cases(sh, "st_inplace_fma"):
        a = z.copy()
        orc.st_inplace_fma(3, 4, a, x, y, _r(c["ranges"]), float(c["alpha"]), float(c["beta"]))
        assert_close(a, c["out"], what=f"st_inplace_fma {c['ranges'].tolist()}")


def test_left_hs_mul(orc, sh):
    x, y, init = sh["inputs/x"], sh["inputs/y"], sh["inputs/init"]
    for c in shuffle_cases(sh, "left_hs_mul"):
        out = init.copy()
        orc.left_hs_mul(3, 4, out, x, y, _r(c["ranges"]), float(c["beta"]))
        assert_close(out, c["out"], what=f"left_hs_mul {c['ranges'].tolist()}")


def test_adjoints(orc, sh):
    x, y, init = sh["inputs/x"], sh["inputs/y"], sh["inputs/init"]
    for c in shuffle_cases(sh, "st_adj_mul"):
        out = init.copy()
        orc.st_adj_mul(3, 4, out, x, y, _r(c["ranges"]))
        assert_close(out, c["out"], what=f"st_adj_mul {c['ranges'].tolist()}")
    for c in shuffle_cases(sh, "left_hs_adj_lmul"):
        o, f, a = _r(c["ranges"])
        out = init.copy()
        orc.left_hs_adjoint(3, 4, True, out, x, y, (o, f, a))
        assert_close(out, c["out"], what=f"left_hs_adj_lmul {c['ranges'].tolist()}")
    for c in shuffle_cases(sh, "left_hs_adj_rmul"):
        o, f, a = _r(c["ranges"])
        out = init.copy()
        orc.left_hs_adjoint(3, 4, False, out, y, x, (o, a, f))
        assert_close(out, c["out"], what=f"left_hs_adj_rmul {c['ranges'].tolist()}")


def test_tensor_pairing(orc, sh):
    x, y = sh["inputs/x"], sh["inputs/y"]
    for c in shuffle_cases(sh, "tensor_pairing"):
        assert_close(orc.tensor_pairing(3, 4, x, y, _r(c["ranges"])), c["out"], what="tensor_pairing")


@pytest.mark.parametrize("W,D", [(1, 4), (2, 2), (4, 0)])
def test_small_bases(orc, sh, W, D):
    key = f"small_{W}_{D}"
    a, b, init = sh[f"{key}/a"], sh[f"{key}/b"], sh[f"{key}/init"]
    full = ((0, D),) * 3
    for name in ("st_mul", "left_hs_mul", "st_adj_mul", "left_hs_adj_lmul", "left_hs_adj_rmul"):
        out = init.copy()
        if name.startswith("left_hs_adj"):
            orc.left_hs_adjoint(W, D, name.endswith("lmul"), out, a, b, full)
        else:
            getattr(orc, name)(W, D, out, a, b, full)
        assert_close(out, sh[f"{key}/{name}"], what=f"{name} W{W} D{D}")


def test_shuffle_is_commutative_and_unit_preserving(orc):
    """x sh y = y sh x, and 1 sh x = x (the empty word is the unit)."""
    W, D = 3, 4
    dim = 121
    rng = np.random.default_rng(4)
    x, y = rng.uniform(-1, 1, (3, dim)), rng.uniform(-1, 1, (3, dim))
    full = ((0, D),) * 3
    xy, yx = np.zeros_like(x), np.zeros_like(x)
    orc.st_mul(W, D, xy, x, y, full)
    orc.st_mul(W, D, yx, y, x, full)
    assert_close(xy, yx, what="commutativity")
    one = np.zeros_like(x)
    one[:, 0] = 1.0
    orc.st_mul(W, D, xy, one, x, full)
    assert_close(xy, x, what="unit")
