"""A thin torch.autograd.Function over the C ABI (the library itself stays
torch-free): forward = rpp_gb_signature, backward = rpp_gb_signature_backward
(reverse pass that recomputes prefixes with exp(-dx)).  Gradchecked against
central finite differences, and compared with the oracle's stored-prefix
adjoint path."""
import importlib

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F64, assert_close

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


class Signature(torch.autograd.Function):
    """S(x) for a batch of equal-length paths; increments [B*L, W]."""

    @staticmethod
    def forward(ctx, incr, basis, length):
        B = incr.shape[0] // length
        st = pkg.GB300Strategy(incr.dtype, incr.device.index or 0)
        sig = torch.empty(B, basis.size(), dtype=incr.dtype, device=incr.device)
        pkg.signature(st, None, incr.contiguous(), basis, B, length=length, out=sig).raise_if_failed()
        ctx.save_for_backward(incr, sig)
        ctx.basis, ctx.length = basis, length
        return sig

    @staticmethod
    def backward(ctx, gsig):
        incr, sig = ctx.saved_tensors
        B = incr.shape[0] // ctx.length
        st = pkg.GB300Strategy(incr.dtype, incr.device.index or 0)
        grad = torch.empty_like(incr)
        pkg.signature_backward(st, None, incr.contiguous(), ctx.basis, B, sig, gsig.contiguous(), grad,
                               length=ctx.length).raise_if_failed()
        return grad, None, None


@pytest.mark.parametrize("W,D,B,L", [(2, 3, 2, 4), (3, 3, 2, 5), (2, 5, 1, 6)])
def test_gradcheck_against_finite_differences(W, D, B, L):
    basis = pkg.TensorBasis(W, D)
    g = torch.Generator(device="cuda").manual_seed(W * 10 + D)
    incr = (torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=g) * 0.4).requires_grad_()
    assert torch.autograd.gradcheck(lambda x: Signature.apply(x, basis, L), (incr,), eps=1e-6, atol=1e-7,
                                    rtol=1e-6)


def test_backward_matches_stored_prefix_path(orc):
    """Loss sum_b <ell_b, S(x_b)> at the differentiation workload's shape,
    scaled down (W6 D4, 16 paths of 128 steps): autograd through the binding
    vs the oracle's stored-prefix adjoint composition."""
    W, D, B, L = 6, 4, 16, 128
    basis = pkg.TensorBasis(W, D)
    rng = np.random.default_rng(21)
    incr_h = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    ell_h = rng.uniform(-1, 1, (B, basis.size()))
    incr = torch.from_numpy(incr_h).cuda().requires_grad_()
    ell = torch.from_numpy(ell_h).cuda()
    loss = (Signature.apply(incr, basis, L) * ell).sum()
    loss.backward()
    _, egrad = orc.signature(W, D, incr_h, np.arange(B + 1) * L, ell=ell_h)
    assert_close(incr.grad.cpu().numpy(), egrad, TOL_F64, "autograd vs stored-prefix adjoint")
