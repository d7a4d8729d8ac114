"""Log-signatures: signature -> ft_log -> tensor_to_lie (one SpMM launch over
the batch), as in the reference's pipeline (include/rpp/operations/
intermediate/ft_log.hpp, include/rpp/operations/basic/tensor_to_lie.hpp)."""
import importlib

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F64, assert_close

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


def logsig(W, D, incr, B, L, dtype=torch.float64):
    basis, lbasis = pkg.TensorBasis(W, D), pkg.LieBasis(W, D)
    dim, ts = basis.size(), lbasis.true_size()
    st = pkg.GB300Strategy(dtype)
    sig = torch.empty(B, dim, dtype=dtype, device="cuda")
    log = torch.empty_like(sig)
    lie = torch.full((B, ts), float("nan"), dtype=dtype, device="cuda")
    assert pkg.signature(st, None, incr, basis, B, length=L, out=sig)
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    assert pkg.ft_log(st, None, full(log), full(sig), basis, B)
    t2l = pkg.make_t2l_matrix(lbasis)
    assert pkg.tensor_to_lie(st, None, pkg.make_lie_batch(lie, ts, 1, D), full(log), lbasis, basis, B, t2l)
    return basis, lbasis, sig, log, lie


@pytest.mark.parametrize("W,D", [(5, 5), (2, 6), (16, 3)])
def test_log_signature_matches_oracle(orc, W, D):
    B, L = 12, 48
    rng = np.random.default_rng(W + D)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    basis, lbasis, sig, log, lie = logsig(W, D, torch.from_numpy(incr).cuda(), B, L)
    esig, _ = orc.signature(W, D, incr, np.arange(B + 1) * L)
    elog = np.zeros_like(esig)
    orc.ft_log(W, D, elog, esig, ((0, D), (0, D)))
    tab = O.LieTables(W, D)
    off, idx, val, _ = tab.t2l_csc()
    elie = np.full((B, tab.true_size), np.nan)
    orc.spmv(True, off, idx, val, elie, 1, tab.true_size - 1, elog, 0)
    torch.cuda.synchronize()
    assert_close(log.cpu().numpy(), elog, TOL_F64, "ft_log of signatures")
    got = lie.cpu().numpy()
    assert np.isnan(got[:, 0]).all()
    assert_close(got[:, 1:], elie[:, 1:], TOL_F64, "log-signature in the Hall basis")


def test_log_signature_roundtrip_full_size():
    """4096 paths, W5 D5, L 256: the log-signature is a Lie element, so
    lie_to_tensor(tensor_to_lie(log S)) = log S, and log S has no degree-0 part."""
    W, D, B, L = 5, 5, 4096, 256
    g = torch.Generator(device="cuda").manual_seed(9)
    incr = torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=g) / np.sqrt(L)
    basis, lbasis, sig, log, lie = logsig(W, D, incr, B, L)
    dim, ts = basis.size(), lbasis.true_size()
    st = pkg.GB300Strategy(torch.float64)
    back = torch.full_like(log, float("nan"))
    l2t = pkg.make_l2t_matrix(lbasis)
    assert pkg.lie_to_tensor(st, None, pkg.make_tensor_batch(back, dim, 0, D), pkg.make_lie_batch(lie, ts, 1, D),
                             basis, lbasis, B, l2t)
    torch.cuda.synchronize()
    assert_close(back.cpu().numpy(), log.cpu().numpy(), TOL_F64, "l2t(t2l(log S)) = log S")
    assert float(log[:, 0].abs().max()) == 0.0
