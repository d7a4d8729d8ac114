"""Ragged batches: paths of uneven length in one launch (longest-first work
counter), and the uneven-length workload captured in a CUDA graph in FP64 and
FP32."""
import importlib

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F32, TOL_F64, assert_close, rel_err, scaled_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


def ragged(rng, n, lo, hi, W):
    lengths = rng.integers(lo, hi + 1, n)
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = rng.normal(0, 1, (offsets[-1], W)) / np.sqrt(np.repeat(np.maximum(lengths, 1), lengths))[:, None]
    return lengths, offsets, incr


@pytest.mark.parametrize("dtype,tol", [(torch.float64, TOL_F64), (torch.float32, TOL_F32)])
def test_ragged_parity_against_oracle(orc, dtype, tol):
    W, D = 8, 4
    rng = np.random.default_rng(31)
    lengths, offsets, incr = ragged(rng, 300, 0, 120, W)
    lengths[::37] = 1
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = rng.normal(0, 0.1, (offsets[-1], W))
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    ell = rng.uniform(-1, 1, (len(lengths), dim))
    st = pkg.GB300Strategy(dtype)
    sig = torch.empty(len(lengths), dim, dtype=dtype, device="cuda")
    grad = torch.empty(incr.shape, dtype=dtype, device="cuda")
    assert pkg.signature(st, None, torch.from_numpy(incr).to("cuda", dtype), basis, len(lengths),
                         offsets=torch.from_numpy(offsets).cuda(), out=sig,
                         seed=torch.from_numpy(ell).to("cuda", dtype), grad=grad)
    torch.cuda.synchronize()
    esig, egrad = orc.signature(W, D, incr, offsets, ell=ell)
    assert_close(sig.double().cpu().numpy(), esig, tol, "ragged signature")
    g = grad.double().cpu().numpy()
    e = scaled_err(g, egrad)
    assert e <= tol, f"ragged gradient: scaled error {e:.3e}"


def test_uneven_workload_in_cuda_graph(orc):
    """10,000 paths, lengths U{16..2048}, W8 D4, increments N(0, 1/len): one
    persistent launch per precision, both captured in one CUDA graph; replays
    equal the eager results bit for bit, FP64 matches the oracle on sampled
    paths, and FP32 is within 1e-5 of FP64 on every coefficient of every path
    (the FP64 results being the oracle's to 1e-12, as the sampled paths show)."""
    W, D, B = 8, 4, 10_000
    rng = np.random.default_rng(2024)
    lengths, offsets, incr = ragged(rng, B, 16, 2048, W)
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    off_d = torch.from_numpy(offsets).cuda()
    x64 = torch.from_numpy(incr).cuda()
    x32 = x64.float()
    st64, st32 = pkg.GB300Strategy(torch.float64), pkg.GB300Strategy(torch.float32)
    s64 = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    s32 = torch.empty(B, dim, dtype=torch.float32, device="cuda")

    def run():
        pkg.signature(st64, None, x64, basis, B, offsets=off_d, out=s64).raise_if_failed()
        pkg.signature(st32, None, x32, basis, B, offsets=off_d, out=s32).raise_if_failed()

    run()
    torch.cuda.synchronize()
    eager64, eager32 = s64.clone(), s32.clone()
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            run()
    torch.cuda.current_stream().wait_stream(stream)
    s64.zero_()
    s32.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(s64, eager64) and torch.equal(s32, eager32)
    pick = np.array([int(np.argmax(lengths)), int(np.argmin(lengths)), 17])
    for b in pick:
        esig, _ = orc.signature(W, D, incr[offsets[b]:offsets[b + 1]], np.array([0, lengths[b]]))
        assert_close(s64[b].cpu().numpy()[None], esig, TOL_F64, f"path {b} (length {lengths[b]})")
    err32 = rel_err(s32.double().cpu().numpy(), s64.cpu().numpy())
    assert err32 <= TOL_F32, f"fp32 against fp64: relative error {err32:.3e}"
