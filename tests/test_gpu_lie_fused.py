"""The fused steps either side of the signature, against the oracle and the
unfused composition they replace:

* rpp_gb_log_to_lie = ft_log (include/rpp/operations/intermediate/ft_log.hpp)
  then tensor_to_lie (include/rpp/operations/basic/tensor_to_lie.hpp);
* rpp_gb_lie_to_tensor_exp = lie_to_tensor (include/rpp/operations/basic/
  lie_to_tensor.hpp) then ft_exp / ft_fmexp (include/rpp/operations/
  intermediate/ft_exp.hpp, ft_fmexp.hpp).

W6 D6 states exceed shared memory, so that shape runs the composed path."""
import importlib

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F32, TOL_F64, assert_close

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")

SHAPES = [(5, 5, 16), (2, 6, 8), (16, 3, 8), (4, 4, 32), (6, 6, 2), (2, 12, 3)]


def _setup(W, D):
    basis, lbasis = pkg.TensorBasis(W, D), pkg.LieBasis(W, D)
    return basis, lbasis, basis.size(), lbasis.true_size()


@pytest.mark.parametrize("W,D,B", SHAPES)
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_log_to_lie_matches_oracle_and_composition(orc, W, D, B, dtype):
    basis, lbasis, dim, ts = _setup(W, D)
    rng = np.random.default_rng(W * 10 + D)
    # group-like arguments: exp of a small random tensor, so log is well posed
    small = rng.uniform(-0.3, 0.3, (B, dim))
    small[:, 0] = 0.0
    x = np.zeros((B, dim))
    orc.ft_exp(W, D, x, small, ((0, D), (0, D)))
    log = np.zeros_like(x)
    orc.ft_log(W, D, log, x, ((0, D), (0, D)))
    tab = O.LieTables(W, D)
    off, idx, val, _ = tab.t2l_csc()
    want = np.full((B, ts), np.nan)
    orc.spmv(True, off, idx, val, want, 1, ts - 1, log, 0, alpha=0.5)
    st = pkg.GB300Strategy(dtype)
    xd = torch.from_numpy(x).to("cuda", dtype)
    got = torch.full((B, ts), float("nan"), dtype=dtype, device="cuda")
    t2l = pkg.make_t2l_matrix(lbasis)
    lb = pkg.make_lie_batch(got, ts, 1, D)
    assert pkg.tensor_log_to_lie(st, None, lb, pkg.make_tensor_batch(xd, dim, 0, D), lbasis, basis, B, t2l,
                                 alpha=0.5)
    # the unfused composition on the same inputs
    logd = torch.empty_like(xd)
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    comp = torch.full_like(got, float("nan"))
    assert pkg.ft_log(st, None, full(logd), full(xd), basis, B)
    assert pkg.sparse_matrix_vector_product(st, None, pkg.make_lie_batch(comp, ts, 1, D), full(logd), lbasis,
                                            basis, B, t2l, alpha=0.5)
    torch.cuda.synchronize()
    tol = TOL_F64 if dtype == torch.float64 else TOL_F32
    g = got.double().cpu().numpy()
    assert np.isnan(g[:, 0]).all(), "wrote outside the Lie view"
    assert_close(g[:, 1:], want[:, 1:], tol, f"log_to_lie W{W} D{D}")
    assert_close(g[:, 1:], comp.double().cpu().numpy()[:, 1:], tol, "fused vs composed")


@pytest.mark.parametrize("W,D,B", SHAPES)
@pytest.mark.parametrize("with_multiplier", [False, True])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_lie_to_tensor_exp_matches_oracle(orc, W, D, B, with_multiplier, dtype):
    basis, lbasis, dim, ts = _setup(W, D)
    rng = np.random.default_rng(W * 7 + D)
    lam = rng.uniform(-0.5, 0.5, (B, ts))
    lam[:, 0] = 0.0
    tab = O.LieTables(W, D)
    off, idx, val, _ = tab.l2t_csc()
    X = np.zeros((B, dim))
    orc.spmv(True, off, idx, val, X, 0, dim, lam, 1, alpha=0.75)
    mult = rng.uniform(-1, 1, (B, dim)) if with_multiplier else None
    want = np.full((B, dim), np.nan)
    if with_multiplier:
        orc.ft_fmexp(W, D, want, mult, X, ((0, D), (0, D), (0, D)))
    else:
        orc.ft_exp(W, D, want, X, ((0, D), (0, D)))
    st = pkg.GB300Strategy(dtype)
    lamd = torch.from_numpy(lam).to("cuda", dtype)
    out = torch.full((B, dim), float("nan"), dtype=dtype, device="cuda")
    l2t = pkg.make_l2t_matrix(lbasis)
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    mb = full(torch.from_numpy(mult).to("cuda", dtype)) if with_multiplier else None
    assert pkg.lie_to_tensor_exp(st, None, full(out), mb, pkg.make_lie_batch(lamd, ts, 1, D), basis, lbasis, B,
                                 l2t, alpha=0.75)
    torch.cuda.synchronize()
    tol = TOL_F64 if dtype == torch.float64 else TOL_F32
    assert_close(out.double().cpu().numpy(), want, tol, f"lie_to_tensor_exp W{W} D{D} mult={with_multiplier}")


def test_partial_views_and_errors():
    """A tensor view starting above degree 0 (the matrix then maps onto
    degrees [1, D]); shape checks are refused before any launch."""
    W, D, B = 3, 4, 4
    basis, lbasis, dim, ts = _setup(W, D)
    st = pkg.GB300Strategy(torch.float64)
    l2t = pkg.make_l2t_matrix(lbasis)
    lam = torch.zeros(B, ts, dtype=torch.float64, device="cuda")
    out = torch.zeros(B, dim, dtype=torch.float64, device="cuda")
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    # the l2t matrix has one row per tensor coefficient: a view without
    # degree 0 is one row short and must be refused
    err = pkg.lie_to_tensor_exp(st, None, full(out), None, pkg.make_lie_batch(lam, ts, 1, D), basis, lbasis, B,
                                l2t, tensor_degrees=(1, D))
    assert not err and err.code == pkg.ErrorCode.OutOfBounds
    err = pkg.lie_to_tensor_exp(st, None, full(out), None, pkg.make_lie_batch(lam, ts, 1, D), basis, lbasis, B,
                                l2t, tensor_degrees=(3, 2))
    assert not err and err.code == pkg.ErrorCode.InvalidArgument


def test_exp_log_roundtrip_full_size():
    """4096 Lie elements of W5 D5: t2l(log(exp(l2t(lambda)))) = lambda through
    the two fused kernels (exp and log are inverse on Lie elements)."""
    W, D, B = 5, 5, 4096
    basis, lbasis, dim, ts = _setup(W, D)
    st = pkg.GB300Strategy(torch.float64)
    g = torch.Generator(device="cuda").manual_seed(3)
    lam = (torch.rand(B, ts, dtype=torch.float64, device="cuda", generator=g) - 0.5) * 0.6
    lam[:, 0] = 0.0
    out = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    back = torch.full_like(lam, float("nan"))
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    assert pkg.lie_to_tensor_exp(st, None, full(out), None, pkg.make_lie_batch(lam, ts, 1, D), basis, lbasis, B,
                                 pkg.make_l2t_matrix(lbasis))
    assert pkg.tensor_log_to_lie(st, None, pkg.make_lie_batch(back, ts, 1, D), full(out), lbasis, basis, B,
                                 pkg.make_t2l_matrix(lbasis))
    torch.cuda.synchronize()
    assert_close(back[:, 1:].cpu().numpy(), lam[:, 1:].cpu().numpy(), 1e-11, "log(exp(lambda)) = lambda")
