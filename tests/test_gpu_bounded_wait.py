"""Bounded waits of the bulk-copy staging (rough-path-primitives_gb300/csrc/
bulk_stage.cuh): operations leave the plan's fault word at zero; a one-CTA
self-test whose wait nothing completes expires after a short limit, records
the fault and returns (no GPU fault, no hang), and reading the word clears
it.  Also the staged paths with rows that start off the 16-byte grid (odd
strides and offsets), whose ends are copied by plain loads."""
import ctypes
import importlib

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F64, assert_close

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


def _fault(plan):
    word = ctypes.c_uint32(12345)
    assert pkg.library().rpp_gb_plan_fault(plan, ctypes.byref(word)) == 0
    return word.value


def test_fault_word_and_expired_wait_self_test():
    basis = pkg.TensorBasis(4, 4)
    plan = basis.plan(0)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    x = torch.rand(64, dim, dtype=torch.float64, device="cuda")
    out = torch.empty_like(x)
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, 4)  # noqa: E731
    assert pkg.ft_mul(st, None, full(out), full(x), full(x), basis, 64)
    assert pkg.st_adj_mul(st, None, full(out), full(x), full(x), basis, 64)
    assert _fault(plan) == 0
    lib = pkg.library()
    assert lib.rpp_gb_selftest_bounded_wait(plan, torch.cuda.current_stream().cuda_stream) == 0
    assert _fault(plan) == 1
    assert _fault(plan) == 0
    # the context is still usable
    assert pkg.ft_mul(st, None, full(out), full(x), full(x), basis, 64)
    torch.cuda.synchronize()
    assert _fault(plan) == 0


@pytest.mark.parametrize("stride_pad,offset", [(0, 0), (1, 1), (3, 2), (5, 7)])
def test_unaligned_rows(orc, stride_pad, offset):
    """Rows at odd element offsets and strides: the bulk copy takes the 16-byte
    aligned interior, plain loads take the ends."""
    W, D, B = 3, 4, 9
    dim = O.tensor_dim(W, D)
    stride = dim + stride_pad
    rng = np.random.default_rng(stride_pad * 10 + offset)
    buf_a = rng.uniform(-1, 1, offset + B * stride)
    buf_b = rng.uniform(-1, 1, offset + B * stride)
    a = np.lib.stride_tricks.as_strided(buf_a[offset:], (B, dim), (stride * 8, 8)).copy()
    b = np.lib.stride_tricks.as_strided(buf_b[offset:], (B, dim), (stride * 8, 8)).copy()
    rr = ((0, D), (1, 3), (0, D))
    want = np.zeros((B, dim))
    orc.ft_mul(W, D, want, a, b, rr)
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float64)
    da = torch.from_numpy(buf_a).cuda()
    db = torch.from_numpy(buf_b).cuda()
    out = torch.zeros(B, dim, dtype=torch.float64, device="cuda")
    la = pkg.make_tensor_batch(da, stride, *rr[1], offset=offset)
    lb = pkg.make_tensor_batch(db, stride, *rr[2], offset=offset)
    assert pkg.ft_mul(st, None, pkg.make_tensor_batch(out, dim, 0, D), la, lb, basis, B)
    torch.cuda.synchronize()
    assert_close(out.cpu().numpy(), want, TOL_F64, f"ft_mul stride {stride} offset {offset}")
    # the shuffle product and adjoint kernels stage the same way
    want = np.zeros((B, dim))
    orc.st_adj_mul(W, D, want, a, b, rr)
    out.zero_()
    assert pkg.st_adj_mul(st, None, pkg.make_tensor_batch(out, dim, 0, D), la, lb, basis, B)
    torch.cuda.synchronize()
    assert_close(out.cpu().numpy(), want, TOL_F64, f"st_adj_mul stride {stride} offset {offset}")
    assert _fault(basis.plan(0)) == 0


def test_sparse_fault_word_stays_clear():
    W, D, B = 4, 4, 16
    basis, lbasis = pkg.TensorBasis(W, D), pkg.LieBasis(W, D)
    dim, ts = basis.size(), lbasis.true_size()
    st = pkg.GB300Strategy(torch.float64)
    x = torch.rand(B, dim, dtype=torch.float64, device="cuda")
    lie = torch.empty(B, ts, dtype=torch.float64, device="cuda")
    t2l = pkg.make_t2l_matrix(lbasis)
    assert pkg.tensor_to_lie(st, None, pkg.make_lie_batch(lie, ts, 1, D), pkg.make_tensor_batch(x, dim, 0, D),
                             lbasis, basis, B, t2l)
    word = ctypes.c_uint32(7)
    assert pkg.library().rpp_gb_matrix_fault(t2l.handle(0), ctypes.byref(word)) == 0
    assert word.value == 0
