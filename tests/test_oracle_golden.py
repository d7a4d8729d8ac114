"""The CPU oracle reproduces the reference's own outputs (golden fixtures
generated by tests/golden/make_golden.py from the unmodified reference)."""
import json
import os

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F64, assert_close

OPS_FILE = "ops_w3d4.npz"


def _cases(z, op):
    keys = sorted({k.split("/")[1] for k in z.files if k.startswith(op + "/")}, key=int)
    return [{k.split("/")[2]: z[k] for k in z.files if k.startswith(f"{op}/{i}/")} for i in keys]


@pytest.fixture(scope="module")
def ops(golden_dir):
    return np.load(os.path.join(golden_dir, OPS_FILE))


def _r(ranges):
    return tuple(tuple(int(v) for v in r) for r in ranges)


def test_ft_mul(orc, ops):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, "ft_mul"):
        out = c["init"].copy()
        orc.ft_mul(W, D, out, c["lhs"], c["rhs"], _r(c["ranges"]), float(c["beta"]))
        assert_close(out, c["out"], what=f"ft_mul {c['ranges'].tolist()}")


def test_ft_fma(orc, ops):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, "ft_fma"):
        out = c["init"].copy()
        orc.ft_fma(W, D, out, c["a"], c["b"], c["c"], _r(c["ranges"]), float(c["alpha"]), float(c["beta"]))
        assert_close(out, c["out"], what=f"ft_fma {c['ranges'].tolist()}")


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_ft_inplace_fma(orc, ops, kind):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, f"ft_inplace_fma{kind}"):
        a = c["a"].copy()
        orc.ft_inplace_fma(W, D, kind, a, c["b"], c["c"], _r(c["ranges"]), float(c["alpha"]), float(c["beta"]))
        assert_close(a, c["out"], what=f"inplace_fma{kind} {c['ranges'].tolist()}")


def test_ft_inplace_mul(orc, ops):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, "ft_inplace_mul"):
        a = c["a"].copy()
        orc.ft_inplace_mul(W, D, a, c["b"], _r(c["ranges"]), float(c["beta"]))
        assert_close(a, c["out"], what=f"inplace_mul {c['ranges'].tolist()}")


@pytest.mark.parametrize("op", ["ft_exp", "ft_log"])
def test_exp_log(orc, ops, op):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, op):
        out = c["init"].copy()
        getattr(orc, op)(W, D, out, c["arg"], _r(c["ranges"]))
        assert_close(out, c["out"], what=f"{op} {c['ranges'].tolist()}")


def test_ft_fmexp(orc, ops):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, "ft_fmexp"):
        out = c["init"].copy()
        orc.ft_fmexp(W, D, out, c["mult"], c["x"], _r(c["ranges"]))
        assert_close(out, c["out"], what=f"fmexp {c['ranges'].tolist()}")


@pytest.mark.parametrize("left", [1, 0])
def test_adjoints(orc, ops, left):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, "ft_adj_lmul" if left else "ft_adj_rmul"):
        out = c["init"].copy()
        orc.ft_adj_mul(W, D, left, out, c["op"], c["arg"], _r(c["ranges"]))
        assert_close(out, c["out"], what=f"adj left={left} {c['ranges'].tolist()}")


@pytest.mark.parametrize("signed", [1, 0])
def test_antipode_bit_exact(orc, ops, signed):
    W, D = int(ops["width"]), int(ops["depth"])
    for c in _cases(ops, "tensor_antipode" if signed else "tensor_reflect"):
        out = c["init"].copy()
        orc.antipode(W, D, signed, out, c["arg"], _r(c["ranges"]))
        assert np.array_equal(out, c["out"])


@pytest.mark.parametrize("wd", [(3, 4), (4, 4), (5, 5), (2, 6)])
def test_lie_tables_bit_exact(golden_dir, wd):
    z = np.load(os.path.join(golden_dir, f"lie_{wd[0]}_{wd[1]}.npz"))
    tab = O.LieTables(*wd)
    assert tab.db == z["degree_begin"].tolist()
    assert tab.pairs == [tuple(p) for p in z["pairs"].tolist()]
    for name, mine in (("t2l", tab.t2l_csc()), ("l2t", tab.l2t_csc())):
        assert np.array_equal(mine[0], z[f"{name}_offsets"])
        assert np.array_equal(mine[1], z[f"{name}_indices"])
        assert np.array_equal(mine[2], z[f"{name}_values"])  # bit-exact values too
        assert tuple(mine[3]) == tuple(z[f"{name}_dims"].tolist())


@pytest.mark.parametrize("wd", [(3, 4), (5, 5)])
def test_lie_conversions(orc, golden_dir, wd):
    z = np.load(os.path.join(golden_dir, f"lie_{wd[0]}_{wd[1]}.npz"))
    W, D = wd
    out = np.full_like(z["t2l_out"], np.nan)
    orc.spmv(True, z["t2l_offsets"], z["t2l_indices"], z["t2l_values"], out, 1, out.shape[1] - 1,
             z["t2l_arg"], 0)
    assert np.isnan(out[:, 0]).all() and np.isnan(z["t2l_out"][:, 0]).all()
    assert_close(out[:, 1:], z["t2l_out"][:, 1:], what="tensor_to_lie")
    out = np.full_like(z["l2t_out"], np.nan)
    orc.spmv(True, z["l2t_offsets"], z["l2t_indices"], z["l2t_values"], out, 0, out.shape[1],
             z["l2t_arg"], 1)
    assert_close(out, z["l2t_out"], what="lie_to_tensor")


def test_signature(orc, golden_dir):
    z = np.load(os.path.join(golden_dir, "signature_w4d4.npz"))
    sig, _ = orc.signature(int(z["width"]), int(z["depth"]), z["incr"], z["offsets"])
    assert_close(sig, z["sig"], what="signature")


def test_kats(orc, golden_dir):
    with open(os.path.join(golden_dir, "kat.json")) as f:
        kat = json.load(f)
    for W, deg, idx, expect in kat["reverse_index"]:
        assert orc.reverse_index(W, deg, idx) == expect
    for W, D, left, right, hint, expect in kat["find_bracket"]:
        assert O.LieTables(W, D).find_bracket(left, right) == expect


def test_gradient_matches_finite_differences(orc):
    rng = np.random.default_rng(5)
    W, D, B, L = 3, 3, 2, 4
    incr = rng.normal(0, 0.5, (B * L, W))
    offs = np.arange(B + 1) * L
    ell = rng.uniform(-1, 1, (B, O.tensor_dim(W, D)))
    _, g = orc.signature(W, D, incr, offs, ell=ell)
    h = 1e-6
    fd = np.zeros_like(incr)
    for i in range(incr.shape[0]):
        for a in range(W):
            p, m = incr.copy(), incr.copy()
            p[i, a] += h
            m[i, a] -= h
            fd[i, a] = ((orc.signature(W, D, p, offs)[0] - orc.signature(W, D, m, offs)[0]) * ell).sum() / (2 * h)
    assert np.max(np.abs(g - fd)) < 1e-7


@pytest.mark.skipif(not os.path.exists(O.REF_LIB_PATH),
                    reason="the reference's headers are not installed (oracle/_ref not built)")
@pytest.mark.parametrize("W,D,lengths", [(3, 4, (5, 0, 17, 1)), (5, 5, (32, 9)), (2, 6, (11, 3, 7))])
def test_reference_reverse_pass_matches_oracle(orc, W, D, lengths):
    """The reference's own forward and stored-prefix reverse pass (its CPU
    strategy driven through rpp::ops in oracle/_ref) against the oracle's
    restatement, on ragged batches with empty and unit paths: the two CPU arms
    the benchmark may time compute the same thing."""
    ref = O.RefBridge()
    rng = np.random.default_rng(W * 10 + D)
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = rng.normal(0, 0.3, (int(offsets[-1]), W))
    ell = rng.uniform(-1, 1, (len(lengths), O.tensor_dim(W, D)))
    rs, rg = ref.signature(W, D, incr, offsets, ell=ell, threads=2)
    es, eg = orc.signature(W, D, incr, offsets, ell=ell)
    assert_close(rs, es, TOL_F64, "reference signature")
    assert_close(rg, eg, TOL_F64, "reference gradient")
