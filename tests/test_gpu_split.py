"""States split over a thread-block cluster (schedule bits 28-30 = P - 1: P
CTAs per path, each holding the coefficients of one range of first letters, the letter
gradients exchanged through distributed shared memory) against the oracle:
forward + reverse, forward only, gradient only, ragged batches with empty and
unit paths, top level in shared or in global memory, FP64 at 1e-12 and FP32
at 1e-5 of the FP64 oracle."""
import importlib

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F32, TOL_F64, assert_close, scaled_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


def split(P, threads):
    return threads | ((P - 1) << 28)


def run(W, D, incr, schedule, *, offsets=None, length=None, ell=None, dtype=torch.float64, want_sig=True):
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    B = len(offsets) - 1 if offsets is not None else incr.shape[0] // length
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)  # noqa: E731
    sig = torch.full((B, dim), float("nan"), dtype=dtype, device="cuda") if want_sig else None
    seed = dev(ell, dtype) if ell is not None else None
    grad = torch.full(incr.shape, float("nan"), dtype=dtype, device="cuda") if ell is not None else None
    err = pkg.signature(pkg.GB300Strategy(dtype), None, dev(incr, dtype), basis, B, length=length,
                        offsets=None if offsets is None else dev(offsets, torch.int64), out=sig, seed=seed,
                        grad=grad, schedule=schedule)
    assert err, err.message
    torch.cuda.synchronize()
    return (None if sig is None else sig.double().cpu().numpy(),
            None if grad is None else grad.double().cpu().numpy())


def check(orc, W, D, incr, offsets, ell, sig, grad, tol, what):
    esig, egrad = orc.signature(W, D, incr, offsets, ell=ell)
    if sig is not None:
        assert_close(sig, esig, tol, f"{what} signature")
    if grad is not None:
        e = scaled_err(grad, egrad)
        assert e <= tol, f"{what} gradient: scaled error {e:.3e}"


@pytest.mark.parametrize("W,D,P,B,L,threads", [
    (6, 6, 2, 3, 6, 512), (6, 6, 3, 3, 6, 256), (6, 6, 6, 3, 6, 256), (6, 6, 6, 2, 5, 512),
    (2, 12, 2, 3, 10, 256), (2, 12, 2, 2, 7, 512), (4, 5, 2, 5, 12, 256), (4, 5, 4, 5, 12, 256),
    (3, 6, 3, 4, 9, 256), (8, 4, 8, 4, 8, 256), (8, 4, 2, 4, 8, 512),
    # bit 15: the top level in the signature and seed rows
    (6, 6, 6, 3, 6, 256 | (1 << 15)), (4, 5, 4, 5, 12, 128 | (1 << 15)),
    # bit 26: the cotangent level and chains in a global workspace
    (2, 12, 2, 3, 10, 256 | (1 << 26)), (2, 12, 2, 2, 7, 512 | (1 << 15) | (1 << 26)),
    (6, 6, 3, 3, 6, 512 | (1 << 26)), (3, 6, 3, 4, 9, 128 | (1 << 26))])
def test_forward_and_reverse_fp64(orc, W, D, P, B, L, threads):
    rng = np.random.default_rng(W * 1000 + D * 10 + P)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    ell = rng.uniform(-1, 1, (B, O.tensor_dim(W, D)))
    sig, grad = run(W, D, incr, split(P, threads), length=L, ell=ell)
    check(orc, W, D, incr, np.arange(B + 1) * L, ell, sig, grad, TOL_F64, f"W{W} D{D} P{P}")


@pytest.mark.parametrize("W,D,P", [(6, 6, 6), (6, 6, 2), (4, 5, 2)])
def test_forward_only(orc, W, D, P):
    rng = np.random.default_rng(7 * W + D + P)
    B, L = 4, 7
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    sig, _ = run(W, D, incr, split(P, 256), length=L)
    check(orc, W, D, incr, np.arange(B + 1) * L, None, sig, None, TOL_F64, f"W{W} D{D} P{P} forward")


def test_gradient_only(orc):
    W, D, P, B, L = 6, 6, 3, 3, 5
    rng = np.random.default_rng(66)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    ell = rng.uniform(-1, 1, (B, O.tensor_dim(W, D)))
    _, grad = run(W, D, incr, split(P, 256), length=L, ell=ell, want_sig=False)
    check(orc, W, D, incr, np.arange(B + 1) * L, ell, None, grad, TOL_F64, "W6 D6 P3 gradient only")


@pytest.mark.parametrize("W,D,P,cot", [(6, 5, 3, 0), (2, 10, 2, 0), (4, 4, 4, 0), (2, 10, 2, 1 << 26)])
def test_ragged_with_empty_and_unit_paths(orc, W, D, P, cot):
    rng = np.random.default_rng(100 + W * D + P)
    lengths = np.array([0, 1, 13, 2, 0, 9, 1, 21, 5])
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = rng.normal(0, 0.3, (int(offsets[-1]), W))
    ell = rng.uniform(-1, 1, (len(lengths), O.tensor_dim(W, D)))
    sig, grad = run(W, D, incr, split(P, 256) | cot, offsets=offsets, ell=ell)
    check(orc, W, D, incr, offsets, ell, sig, grad, TOL_F64, f"ragged W{W} D{D} P{P}")


@pytest.mark.parametrize("W,D,P", [(6, 6, 3), (2, 12, 2), (8, 4, 4)])
def test_fp32_against_fp64_oracle(orc, W, D, P):
    rng = np.random.default_rng(200 + W + D + P)
    B, L = 3, 8
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    ell = rng.uniform(-1, 1, (B, O.tensor_dim(W, D)))
    sig, grad = run(W, D, incr, split(P, 256), length=L, ell=ell, dtype=torch.float32)
    check(orc, W, D, incr, np.arange(B + 1) * L, ell, sig, grad, TOL_F32, f"FP32 W{W} D{D} P{P}")


def test_split_refuses_what_it_cannot_run():
    """P must divide the width, and the split form is one fused launch."""
    W, D, B, L = 5, 4, 2, 3
    basis = pkg.TensorBasis(W, D)
    x = torch.zeros(B * L, W, dtype=torch.float64, device="cuda")
    sig = torch.empty(B, basis.size(), dtype=torch.float64, device="cuda")
    err = pkg.signature(pkg.GB300Strategy(torch.float64), None, x, basis, B, length=L, out=sig,
                        schedule=split(2, 256))
    assert not err
    torch.cuda.synchronize()
    # the context keeps working
    err = pkg.signature(pkg.GB300Strategy(torch.float64), None, x, basis, B, length=L, out=sig, schedule=256)
    assert err, err.message
