"""Fused signature forward / reverse kernels against the oracle.

The oracle's reverse pass stores every prefix and composes ft_adj_lmul,
ft_adj_rmul and the derivative of the letter-only exponential; the kernel
recomputes prefixes backwards instead.  Tolerances: 1e-12 relative (FP64),
1e-5 (FP32 against the FP64 oracle)."""
import importlib
import os

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F32, TOL_F64, assert_close, rel_err, scaled_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def run(W, D, incr, offsets=None, length=None, ell=None, dtype=torch.float64, want_sig=True):
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    B = len(offsets) - 1 if offsets is not None else incr.shape[0] // length
    sig = torch.full((B, dim), float("nan"), dtype=dtype, device="cuda") if want_sig else None
    seed = dev(ell, dtype) if ell is not None else None
    grad = torch.full(incr.shape, float("nan"), dtype=dtype, device="cuda") if ell is not None else None
    err = pkg.signature(st, None, dev(incr, dtype), basis, B, length=length,
                        offsets=None if offsets is None else dev(offsets, torch.int64), out=sig, seed=seed, grad=grad)
    assert err, err.message
    return (host(sig) if want_sig else None), (host(grad) if grad is not None else None)


def test_golden_signature(golden_dir):
    z = np.load(os.path.join(golden_dir, "signature_w4d4.npz"))
    W, D = int(z["width"]), int(z["depth"])
    L = int(z["offsets"][1])
    sig, _ = run(W, D, z["incr"], length=L)
    assert_close(sig, z["sig"], TOL_F64, "signature vs reference")
    sig32, _ = run(W, D, z["incr"], length=L, dtype=torch.float32)
    assert_close(sig32, z["sig"], TOL_F32, "fp32 signature vs reference")


SHAPES = [(2, 3, 4, 16), (3, 4, 8, 32), (5, 5, 6, 256), (4, 4, 16, 64), (2, 8, 4, 32), (8, 4, 4, 16),
          (16, 3, 2, 8), (1, 4, 3, 5), (3, 1, 5, 7), (6, 6, 2, 8), (2, 12, 2, 16), (7, 3, 3, 9)]


@pytest.mark.parametrize("W,D,B,L", SHAPES)
def test_forward_and_gradient(orc, W, D, B, L):
    rng = np.random.default_rng(W * 31 + D)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    offs = np.arange(B + 1) * L
    esig, egrad = orc.signature(W, D, incr, offs, ell=ell)
    sig, grad = run(W, D, incr, length=L, ell=ell)
    assert_close(sig, esig, TOL_F64, "signature")
    assert_close(grad, egrad, TOL_F64, "gradient")
    sig32, grad32 = run(W, D, incr, length=L, ell=ell, dtype=torch.float32)
    assert_close(sig32, esig, TOL_F32, "fp32 signature against the FP64 oracle")
    e32 = scaled_err(grad32, egrad)
    assert e32 <= TOL_F32, f"fp32 gradient against the FP64 oracle: scaled error {e32:.3e}"


def test_ragged_batch_with_empty_and_unit_paths(orc):
    W, D = 3, 4
    rng = np.random.default_rng(11)
    lengths = np.array([5, 0, 1, 17, 2, 0, 33])
    offs = np.concatenate([[0], np.cumsum(lengths)])
    incr = rng.normal(0, 0.3, (offs[-1], W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (len(lengths), dim))
    esig, egrad = orc.signature(W, D, incr, offs, ell=ell)
    sig, grad = run(W, D, incr, offsets=offs, ell=ell)
    assert_close(sig, esig, TOL_F64, "ragged signature")
    assert_close(grad, egrad, TOL_F64, "ragged gradient")
    unit = np.zeros(dim)
    unit[0] = 1
    assert np.array_equal(sig[1], unit) and np.array_equal(sig[5], unit)


def test_gradient_only_and_backward_entry(orc):
    W, D, B, L = 4, 4, 5, 24
    rng = np.random.default_rng(12)
    incr = rng.normal(0, 0.2, (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    esig, egrad = orc.signature(W, D, incr, np.arange(B + 1) * L, ell=ell)
    _, grad = run(W, D, incr, length=L, ell=ell, want_sig=False)
    assert_close(grad, egrad, TOL_F64, "gradient without signature output")
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float64)
    g = torch.zeros(B * L, W, dtype=torch.float64, device="cuda")
    assert pkg.signature_backward(st, None, dev(incr), basis, B, dev(esig), dev(ell), g, length=L)
    assert_close(host(g), egrad, TOL_F64, "backward from final signatures")


def test_gradient_matches_finite_differences():
    """Central differences (h = 1e-6) of sum_b <ell_b, S(x_b)> computed on the GPU."""
    W, D, B, L = 3, 4, 2, 6
    rng = np.random.default_rng(13)
    incr = rng.normal(0, 0.4, (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    _, grad = run(W, D, incr, length=L, ell=ell)
    h = 1e-6
    fd = np.zeros_like(incr)
    for i in range(incr.shape[0]):
        for a in range(W):
            p, m = incr.copy(), incr.copy()
            p[i, a] += h
            m[i, a] -= h
            sp, _ = run(W, D, p, length=L)
            sm, _ = run(W, D, m, length=L)
            fd[i, a] = ((sp - sm) * ell).sum() / (2 * h)
    assert np.max(np.abs(grad - fd)) < 1e-7


def test_chen_identity_full_size():
    """Size-independent property at the headline shape (W5 D5, 4096 paths of
    256 steps): S(x) = S(first half) (x) S(second half), via the ft_mul kernel,
    and the gradient is linear in the seed."""
    W, D, B, L = 5, 5, 4096, 256
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    g = torch.Generator(device="cuda").manual_seed(5)
    incr = torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=g) / np.sqrt(L)
    full = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    assert pkg.signature(st, None, incr, basis, B, length=L, out=full)
    halves = incr.view(B, 2, L // 2, W)
    first = torch.empty_like(full)
    second = torch.empty_like(full)
    assert pkg.signature(st, None, halves[:, 0].contiguous().view(-1, W), basis, B, length=L // 2, out=first)
    assert pkg.signature(st, None, halves[:, 1].contiguous().view(-1, W), basis, B, length=L // 2, out=second)
    prod = torch.empty_like(full)
    mk = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    assert pkg.ft_mul(st, None, mk(prod), mk(first), mk(second), basis, B)
    assert_close(host(prod), host(full), TOL_F64, "Chen identity")
    ell1 = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    ell2 = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    g1, g2, g12 = (torch.empty_like(incr) for _ in range(3))
    for ell, gg in ((ell1, g1), (ell2, g2), (ell1 + 0.5 * ell2, g12)):
        assert pkg.signature(st, None, incr, basis, B, length=L, seed=ell, grad=gg)
    lin = g1 + 0.5 * g2
    assert_close(host(g12), host(lin), 1e-11, "gradient linearity")


def plain_signature_and_gradient(st, basis, W, D, B, L, incr, ell):
    """The caller's composition of per-operation kernels: the forward pass
    as L ft_fmexp launches with the increments viewed as degree-one tensors
    (tests/rpp/gpu/block/ops/ft_fmexp_tests.cu:126-147), every prefix stored,
    then the reverse pass G_{k-1} = adj_rmul(exp(x_k), G_k) with the increment
    gradient from adj_lmul(S_{k-1}, G_k) through the exp VJP.  `incr` is the
    [B*L, W] device array of one batch of equal-length paths."""
    dim = basis.size()
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    xview = lambda k: pkg.make_tensor_batch(incr, L * W, 1, 1, offset=k * W - 1)  # noqa: E731
    prefixes = torch.empty(L + 1, B, dim, dtype=torch.float64, device="cuda")
    assert pkg.tensor_set_identity(st, None, full(prefixes[0]), basis, B)
    for k in range(L):
        assert pkg.ft_fmexp(st, None, full(prefixes[k + 1]), full(prefixes[k]), xview(k), basis, B)
    G, Gn, H, E = (torch.empty(B, dim, dtype=torch.float64, device="cuda") for _ in range(4))
    grad = torch.full_like(incr, float("nan"))
    G.copy_(ell)
    for k in range(L - 1, -1, -1):
        assert pkg.ft_exp(st, None, full(E), xview(k), basis, B)
        assert pkg.ft_adj_lmul(st, None, full(H), full(prefixes[k]), full(G), basis, B)
        assert pkg.exp_letter_vjp(st, None, H, incr, grad, basis, B, x_stride=L * W, dx_stride=L * W,
                                  x_offset=k * W, dx_offset=k * W)
        assert pkg.ft_adj_rmul(st, None, full(Gn), full(E), full(G), basis, B)
        G, Gn = Gn, G
    return prefixes[L], grad


@pytest.mark.parametrize("W,D,B,L", [(3, 4, 4, 8), (5, 5, 3, 12)])
def test_plain_per_operation_reverse_pass(orc, W, D, B, L):
    """The stored-prefix reverse pass composed from the per-operation kernels
    (ft_fmexp with increments viewed as degree-one tensors, ft_exp, ft_adj_lmul,
    ft_adj_rmul, exp VJP) matches the oracle and the fused kernel."""
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float64)
    rng = np.random.default_rng(W + 7 * D)
    incr_h = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    ell_h = rng.uniform(-1, 1, (B, basis.size()))
    sig, grad = plain_signature_and_gradient(st, basis, W, D, B, L, dev(incr_h), dev(ell_h))
    esig, egrad = orc.signature(W, D, incr_h, np.arange(B + 1) * L, ell=ell_h)
    assert_close(host(sig), esig, TOL_F64, "plain forward")
    assert_close(host(grad), egrad, TOL_F64, "plain reverse")
    fsig, fgrad = run(W, D, incr_h, length=L, ell=ell_h)
    assert_close(fsig, host(sig), TOL_F64, "fused against plain forward")
    assert_close(fgrad, host(grad), TOL_F64, "fused against plain reverse")


def test_gradient_check_width6_depth6_full_batch(orc):
    """Gradient of sum_b <l_b, S(x_b)> at width 6, depth 6 (55 987
    coefficients), 512 paths of 128 increments N(0, 1/128), l_b ~ U[-1, 1]:
    one fused forward + reverse call over the whole batch, checked
    (1) against central differences (h = 1e-6) at 64 random increment
        coordinates -- the 128 perturbed paths run as one forward call;
    (2) against the plain stored-prefix reverse pass of per-operation kernels
        over all 512 paths (in chunks of 64, whose stored prefixes take 3.7 GB);
    (3) against the oracle on three sampled paths."""
    W, D, B, L = 6, 6, 512, 128
    rng = np.random.default_rng(4646)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    sig, grad = run(W, D, incr, length=L, ell=ell)
    assert np.isfinite(sig).all() and np.isfinite(grad).all()

    # (1) central differences
    h = 1e-6
    picks = rng.choice(B * L * W, 64, replace=False)
    rows, letters = picks // W, picks % W
    paths = rows // L
    pert = np.empty((2 * len(picks) * L, W))
    for i, (r, a, b) in enumerate(zip(rows, letters, paths)):
        for sgn, slot in ((1.0, 2 * i), (-1.0, 2 * i + 1)):
            x = incr[b * L:(b + 1) * L].copy()
            x[r - b * L, a] += sgn * h
            pert[slot * L:(slot + 1) * L] = x
    sp, _ = run(W, D, pert, length=L)
    fd = np.array([((sp[2 * i] - sp[2 * i + 1]) * ell[b]).sum() / (2 * h) for i, b in enumerate(paths)])
    got = grad[rows, letters]
    scale = max(1.0, float(np.abs(got).max()))
    fd_err = float(np.max(np.abs(got - fd))) / scale
    assert fd_err < 1e-7, f"gradient against central differences: scaled error {fd_err:.3e}"

    # (2) the plain stored-prefix path over the whole batch
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float64)
    chunk = 64
    for c in range(0, B, chunk):
        psig, pgrad = plain_signature_and_gradient(st, basis, W, D, chunk, L, dev(incr[c * L:(c + chunk) * L]),
                                                   dev(ell[c:c + chunk]))
        assert_close(sig[c:c + chunk], host(psig), TOL_F64, f"paths {c}..: fused against plain forward")
        assert_close(grad[c * L:(c + chunk) * L], host(pgrad), TOL_F64, f"paths {c}..: fused against plain reverse")
        del psig, pgrad
        torch.cuda.empty_cache()

    # (3) the oracle on sampled paths
    for b in (0, 257, B - 1):
        esig, egrad = orc.signature(W, D, incr[b * L:(b + 1) * L], np.array([0, L]), ell=ell[b:b + 1])
        assert_close(sig[b:b + 1], esig, TOL_F64, f"path {b} signature")
        assert_close(grad[b * L:(b + 1) * L], egrad, TOL_F64, f"path {b} gradient")


def test_autotuner_records_schedule_and_keeps_parity(orc):
    W, D, B, L = 4, 4, 64, 32
    rng = np.random.default_rng(41)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float64)
    sig = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    grad = torch.empty(B * L, W, dtype=torch.float64, device="cuda")
    err, threads, ms = pkg.signature_tune(st, None, dev(incr), basis, B, length=L, out=sig, seed=dev(ell), grad=grad)
    assert err, err.message
    # schedule: threads per CTA in bits 0-9, CTA-per-SM cap in bits 10-13,
    # bit 14 for the two-launch form (bit 15: its forward top level in global
    # memory; bits 16-25: its reverse launch's own CTA size), bit 26 for the
    # cotangent arrays in a global workspace, bit 27 for the D-barrier reverse
    # step; no cluster split for a state this small (bits 28-30)
    sizes = (128, 192, 256, 320, 384, 512)
    assert (threads & 1023) in sizes and ((threads >> 10) & 15) in (0, 2, 3)
    assert (threads >> 28) == 0 and ((threads >> 16) & 1023) in (0,) + sizes
    assert ((threads >> 16) & 1023) == 0 or threads & (1 << 14)
    assert ms > 0
    esig, egrad = orc.signature(W, D, incr, np.arange(B + 1) * L, ell=ell)
    assert_close(host(sig), esig, TOL_F64, "tuned signature")
    assert_close(host(grad), egrad, TOL_F64, "tuned gradient")
    sig2, grad2 = run(W, D, incr, length=L, ell=ell)
    assert np.array_equal(sig2, host(sig)) or threads != 0


@pytest.mark.parametrize("schedule", [128, 256, 128 | (3 << 10), 192 | (2 << 10), 128 | (1 << 14),
                                      256 | (1 << 14), 128 | (3 << 14), 320 | (3 << 14),
                                      128 | (1 << 14) | (256 << 16), 256 | (3 << 14) | (128 << 16),
                                      256 | (1 << 26), 128 | (3 << 14) | (1 << 26), 128 | (3 << 14) | (512 << 16) | (1 << 26)])
@pytest.mark.parametrize("ragged", [False, True])
def test_every_schedule_matches_oracle(orc, schedule, ragged):
    """Each schedule the autotuner can pick (CTA size, a cap on CTAs per SM,
    the two-launch form whose reverse launch reads the seed's top level from
    global memory) gives the oracle's signatures and gradients."""
    W, D, B, L = 5, 4, 40, 24
    rng = np.random.default_rng(schedule)
    lengths = rng.integers(0, 2 * L, B) if ragged else np.full(B, L)
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = rng.normal(0, 1 / np.sqrt(L), (int(offsets[-1]), W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    basis = pkg.TensorBasis(W, D)
    sig = torch.full((B, dim), float("nan"), dtype=torch.float64, device="cuda")
    grad = torch.full((int(offsets[-1]), W), float("nan"), dtype=torch.float64, device="cuda")
    incr_d, ell_d = dev(incr), dev(ell)
    off_d = torch.from_numpy(offsets).cuda() if ragged else None
    lib = pkg.library()
    rc = lib.rpp_gb_signature_with_schedule(basis.plan(0), torch.cuda.current_stream().cuda_stream, 1,
                                            incr_d.data_ptr(), None if off_d is None else off_d.data_ptr(),
                                            0 if ragged else L, B, sig.data_ptr(), dim, ell_d.data_ptr(), dim,
                                            grad.data_ptr(), schedule)
    assert rc == 0, lib.rpp_gb_last_error_string()
    torch.cuda.synchronize()
    esig, egrad = orc.signature(W, D, incr, offsets, ell=ell)
    assert_close(host(sig), esig, TOL_F64, f"signature, schedule {schedule}")
    assert_close(host(grad), egrad, TOL_F64, f"gradient, schedule {schedule}")




@pytest.mark.parametrize("schedule", [512 | (1 << 14), 256 | (3 << 14), 128 | (1 << 14) | (512 << 16),
                                      512 | (1 << 14) | (1 << 26), 256 | (1 << 26)])
def test_two_launch_large_state_matches_oracle(orc, schedule):
    """W6 D6 FP64 does not fit shared memory: under a two-launch schedule the
    forward launch keeps its state on chip (top level in global memory) and
    the reverse launch runs in the global workspace -- with 2 x 152 CTAs of
    half size when that workspace fits in L2 -- against the oracle."""
    W, D, B, L = 6, 6, 3, 6
    rng = np.random.default_rng(schedule & 0xFFFF)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    basis = pkg.TensorBasis(W, D)
    sig = torch.full((B, dim), float("nan"), dtype=torch.float64, device="cuda")
    grad = torch.full((B * L, W), float("nan"), dtype=torch.float64, device="cuda")
    err = pkg.signature(pkg.GB300Strategy(torch.float64), None, dev(incr), basis, B, length=L, out=sig,
                        seed=dev(ell), grad=grad, schedule=schedule)
    assert err, err.message
    esig, egrad = orc.signature(W, D, incr, np.arange(B + 1) * L, ell=ell)
    assert_close(host(sig), esig, TOL_F64, f"W6 D6 signature, schedule {schedule}")
    assert_close(host(grad), egrad, TOL_F64, f"W6 D6 gradient, schedule {schedule}")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("schedule", [256 | (3 << 14) | (512 << 16) | (1 << 26), 512 | (1 << 26), 256 | (3 << 14)])
def test_deep_narrow_cotangent_workspace_matches_oracle(orc, schedule, dtype):
    """W2 D12 FP64 (196 KB of reverse state): the cotangent level and chains in
    the global workspace, state and forward chains resident, two CTAs per SM
    -- against the oracle, fused and two-launch."""
    W, D, B, L = 2, 12, 3, 10
    rng = np.random.default_rng(schedule & 0xFFFFF)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim))
    basis = pkg.TensorBasis(W, D)
    sig = torch.full((B, dim), float("nan"), dtype=dtype, device="cuda")
    grad = torch.full((B * L, W), float("nan"), dtype=dtype, device="cuda")
    err = pkg.signature(pkg.GB300Strategy(dtype), None, dev(incr, dtype), basis, B, length=L, out=sig,
                        seed=dev(ell, dtype), grad=grad, schedule=schedule)
    assert err, err.message
    esig, egrad = orc.signature(W, D, incr, np.arange(B + 1) * L, ell=ell)
    tol = TOL_F64 if dtype == torch.float64 else TOL_F32
    assert_close(host(sig), esig, tol, f"W2 D12 signature, schedule {schedule}")
    assert_close(host(grad), egrad, tol, f"W2 D12 gradient, schedule {schedule}")

@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("W,D,B,L,chunk", [(5, 5, 7, 16, 0), (5, 5, 7, 16, 3), (3, 4, 10, 9, 1), (4, 4, 5, 8, 64),
                                           (2, 6, 9, 12, 4)])
def test_host_buffers_equal_device_path(W, D, B, L, chunk, dtype):
    """rpp_gb_signature_host: host tensors in and out, the batch in chunks on
    two internal streams -- bit-identical to the device call (paths are
    independent), with strided host outputs and every output combination."""
    rng = np.random.default_rng(W * 100 + D * 10 + B + chunk)
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    incr = torch.from_numpy(rng.normal(0, 1 / np.sqrt(L), (B * L, W))).to(dtype)
    ell = torch.from_numpy(rng.uniform(-1, 1, (B, dim))).to(dtype)
    want_sig = torch.empty(B, dim, dtype=dtype, device="cuda")
    want_grad = torch.empty(B * L, W, dtype=dtype, device="cuda")
    assert pkg.signature(st, None, incr.cuda(), basis, B, length=L, out=want_sig, seed=ell.cuda(), grad=want_grad)
    torch.cuda.synchronize()
    # strided host signatures (stride dim + 3), contiguous gradients
    sig_h = torch.full((B, dim + 3), float("nan"), dtype=dtype).pin_memory()
    grad_h = torch.full((B * L, W), float("nan"), dtype=dtype).pin_memory()
    seed_h = torch.zeros(B, dim + 2, dtype=dtype)
    seed_h[:, :dim] = ell
    err = pkg.signature_host(st, None, incr.pin_memory(), basis, B, length=L, out=sig_h, out_stride=dim + 3,
                             seed=seed_h.pin_memory(), seed_stride=dim + 2, grad=grad_h, chunk=chunk)
    assert err, err.message
    torch.cuda.synchronize()
    assert torch.equal(sig_h[:, :dim], want_sig.cpu()), "signatures differ from the device path"
    assert torch.isnan(sig_h[:, dim:]).all(), "wrote outside the signature rows"
    assert torch.equal(grad_h, want_grad.cpu()), "gradients differ from the device path"
    # signatures only, then gradients only, each against the device call that
    # asks for the same outputs (a different output set is a different schedule
    # key, and the gradient's reduction order follows the CTA size)
    sig_only = torch.empty(B, dim, dtype=dtype).pin_memory()
    assert pkg.signature_host(st, None, incr, basis, B, length=L, out=sig_only, chunk=chunk)
    grad_only = torch.empty(B * L, W, dtype=dtype)
    assert pkg.signature_host(st, None, incr, basis, B, length=L, seed=ell.contiguous(), grad=grad_only, chunk=chunk)
    only_sig = torch.empty(B, dim, dtype=dtype, device="cuda")
    assert pkg.signature(st, None, incr.cuda(), basis, B, length=L, out=only_sig)
    only_grad = torch.empty(B * L, W, dtype=dtype, device="cuda")
    assert pkg.signature(st, None, incr.cuda(), basis, B, length=L, seed=ell.cuda(), grad=only_grad)
    torch.cuda.synchronize()
    assert torch.equal(sig_only, only_sig.cpu())
    assert torch.equal(grad_only, only_grad.cpu())


def test_host_buffers_refusals():
    basis = pkg.TensorBasis(3, 3)
    st = pkg.GB300Strategy(torch.float64)
    incr = torch.zeros(8, 3, dtype=torch.float64)
    out = torch.zeros(2, basis.size(), dtype=torch.float64)
    err = pkg.signature_host(st, None, incr, basis, 2, length=0, out=out)
    assert not err and err.code == pkg.ErrorCode.InvalidArgument
    with pytest.raises(ValueError):
        pkg.signature_host(st, None, incr.cuda(), basis, 2, length=4, out=out)


@pytest.mark.parametrize("W,D,threads", [(4, 6, 128), (4, 6, 256), (8, 4, 128), (8, 4, 512), (16, 3, 128),
                                         (16, 3, 256), (4, 7, 128), (8, 3, 64)])
@pytest.mark.parametrize("ragged", [False, True])
def test_fp32_forward_top_level_in_registers(orc, W, D, threads, ragged):
    """FP32 forward-only calls with W a multiple of 4 keep the top level's rows
    in registers (8 rows per thread at W = 4, 4 at W = 8, 2 at W = 16; W4 D7
    at 128 threads has more rows than that and keeps the shared-memory form):
    against the FP64 oracle at 1e-5."""
    rng = np.random.default_rng(W * 100 + D * 10 + threads)
    B, L = 9, 11
    if ragged:
        lengths = rng.integers(0, 2 * L, B)
        offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    else:
        offsets = np.arange(B + 1, dtype=np.int64) * L
    incr = rng.normal(0, 1 / np.sqrt(L), (int(offsets[-1]), W))
    basis = pkg.TensorBasis(W, D)
    sig = torch.full((B, basis.size()), float("nan"), dtype=torch.float32, device="cuda")
    err = pkg.signature(pkg.GB300Strategy(torch.float32), None, dev(incr, torch.float32), basis, B,
                        length=None if ragged else L, offsets=dev(offsets, torch.int64) if ragged else None,
                        out=sig, schedule=threads)
    assert err, err.message
    esig, _ = orc.signature(W, D, incr, offsets)
    assert_close(host(sig), esig, TOL_F32, f"FP32 W{W} D{D} forward, {threads} threads")


@pytest.mark.parametrize("W,D", [(8, 4), (8, 2), (5, 5), (5, 3), (4, 5), (6, 4), (3, 6), (16, 2)])
@pytest.mark.parametrize("ragged", [False, True])
def test_fp32_forward_one_warp_per_letter(orc, W, D, ragged):
    """The FP32 forward kernel with one warp per first letter and compile-time
    (width, depth) (schedule bit 16 on a forward-only call): against the FP64
    oracle at 1e-5, equal-length and ragged with empty and unit paths."""
    rng = np.random.default_rng(W * 37 + D)
    B, L = 13, 9
    if ragged:
        lengths = np.array([0, 1, 2, 17, 5, 0, 9, 31, 1, 4, 12, 3, 8])
        offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    else:
        offsets = np.arange(B + 1, dtype=np.int64) * L
    incr = rng.normal(0, 1 / np.sqrt(L), (int(offsets[-1]), W))
    basis = pkg.TensorBasis(W, D)
    sig = torch.full((B, basis.size()), float("nan"), dtype=torch.float32, device="cuda")
    err = pkg.signature(pkg.GB300Strategy(torch.float32), None, dev(incr, torch.float32), basis, B,
                        length=None if ragged else L, offsets=dev(offsets, torch.int64) if ragged else None,
                        out=sig, schedule=32 | (1 << 16))
    assert err, err.message
    esig, _ = orc.signature(W, D, incr, offsets)
    assert_close(host(sig), esig, TOL_F32, f"FP32 letter warps W{W} D{D}")


def test_fp32_one_warp_per_letter_refuses_other_shapes():
    basis = pkg.TensorBasis(7, 4)  # not instantiated
    x = torch.zeros(6, 7, dtype=torch.float32, device="cuda")
    sig = torch.empty(2, basis.size(), dtype=torch.float32, device="cuda")
    err = pkg.signature(pkg.GB300Strategy(torch.float32), None, x, basis, 2, length=3, out=sig,
                        schedule=32 | (1 << 16))
    assert not err


@pytest.mark.parametrize("W,D", [(8, 4), (5, 5), (4, 5), (6, 4), (3, 6)])
def test_fp32_one_warp_per_letter_equals_shared_memory_kernel(W, D):
    """The warp-per-letter kernel forms the same fused multiply-adds in the same
    order as the shared-memory kernel (each chain value recomputed by the lane
    that needs it; x/m rounded once, as the kernel's scaled increments are), so
    the two agree bit for bit."""
    rng = np.random.default_rng(W * 7 + D)
    lengths = rng.integers(0, 40, 21)
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = dev(rng.normal(0, 0.3, (int(offsets[-1]), W)), torch.float32)
    offs = dev(offsets, torch.int64)
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float32)
    out = []
    for schedule in (32 | (1 << 16), 128, 256 | (2 << 10)):
        sig = torch.full((len(lengths), basis.size()), float("nan"), dtype=torch.float32, device="cuda")
        err = pkg.signature(st, None, incr, basis, len(lengths), offsets=offs, out=sig, schedule=schedule)
        assert err, err.message
        out.append(sig)
    torch.cuda.synchronize()
    for k in (1, 2):
        diff = float(torch.max(torch.abs(out[0] - out[k])).item())
        assert torch.equal(out[0], out[k]), f"W{W} D{D}: schedule {k} differs by up to {diff:.3e}"


LETTER_REV_SHAPES = [(8, 4), (5, 5), (5, 3), (4, 5), (6, 4), (3, 6), (8, 3), (4, 4), (3, 5), (5, 4)]


def letter_rev_case(W, D, ragged, seed):
    rng = np.random.default_rng(seed)
    B, L = 13, 9
    if ragged:
        lengths = np.array([0, 1, 2, 17, 5, 0, 9, 31, 1, 4, 12, 3, 8])
        offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    else:
        offsets = np.arange(B + 1, dtype=np.int64) * L
    incr = rng.normal(0, 1 / np.sqrt(L), (int(offsets[-1]), W))
    ell = rng.uniform(-1, 1, (B, O.tensor_dim(W, D)))
    return B, offsets, incr, ell


@pytest.mark.parametrize("W,D", LETTER_REV_SHAPES)
@pytest.mark.parametrize("ragged", [False, True])
def test_fp32_reverse_one_warp_per_letter(orc, W, D, ragged):
    """FP32 forward + reverse with one warp per first letter (schedule bit 16 on
    a call with a reverse pass): signatures and increment gradients against the
    FP64 oracle at 1e-5; ragged batches with empty and unit paths, and lengths
    on both sides of the 8-step blocks in which the letter gradients are added
    across warps."""
    B, offsets, incr, ell = letter_rev_case(W, D, ragged, W * 53 + D)
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float32)
    sig = torch.full((B, basis.size()), float("nan"), dtype=torch.float32, device="cuda")
    grad = torch.full(incr.shape, float("nan"), dtype=torch.float32, device="cuda")
    kw = dict(offsets=dev(offsets, torch.int64)) if ragged else dict(length=int(offsets[1]))
    err = pkg.signature(st, None, dev(incr, torch.float32), basis, B, out=sig, seed=dev(ell, torch.float32),
                        grad=grad, schedule=32 | (1 << 16), **kw)
    assert err, err.message
    esig, egrad = orc.signature(W, D, incr, offsets, ell=ell)
    assert_close(host(sig), esig, TOL_F32, f"FP32 letter warps W{W} D{D} signature")
    e = scaled_err(host(grad), egrad)
    assert e <= TOL_F32, f"FP32 letter warps W{W} D{D} gradient: scaled error {e:.3e}"


@pytest.mark.parametrize("W,D", [(5, 5), (8, 4), (3, 6)])
def test_fp32_reverse_one_warp_per_letter_gradient_only_and_backward_entry(orc, W, D):
    """The same kernel without signature output (its forward pass skips the top
    level) and from given final signatures (rpp_gb_signature_backward, whose
    FP32 calls of these shapes take it without a recorded schedule)."""
    B, offsets, incr, ell = letter_rev_case(W, D, True, W * 59 + D)
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(torch.float32)
    offs = dev(offsets, torch.int64)
    esig, egrad = orc.signature(W, D, incr, offsets, ell=ell)
    grad = torch.full(incr.shape, float("nan"), dtype=torch.float32, device="cuda")
    err = pkg.signature(st, None, dev(incr, torch.float32), basis, B, offsets=offs, seed=dev(ell, torch.float32),
                        grad=grad, schedule=32 | (1 << 16))
    assert err, err.message
    e = scaled_err(host(grad), egrad)
    assert e <= TOL_F32, f"gradient-only W{W} D{D}: scaled error {e:.3e}"
    g2 = torch.full(incr.shape, float("nan"), dtype=torch.float32, device="cuda")
    err = pkg.signature_backward(st, None, dev(incr, torch.float32), basis, B, dev(esig, torch.float32),
                                 dev(ell, torch.float32), g2, offsets=offs)
    assert err, err.message
    e = scaled_err(host(g2), egrad)
    assert e <= TOL_F32, f"backward entry W{W} D{D}: scaled error {e:.3e}"


@pytest.mark.parametrize("W,D", [(5, 5), (8, 4), (4, 5)])
def test_fp32_reverse_one_warp_per_letter_agrees_with_shared_memory_kernel(W, D):
    """The warp-per-letter reverse pass sums the same terms as the shared-memory
    kernel in another order (the letter gradients per slice, then across
    slices): the two agree to a few FP32 roundings, at the headline length."""
    rng = np.random.default_rng(W * 61 + D)
    B, L = 24, 256
    incr = dev(rng.normal(0, 1 / np.sqrt(L), (B * L, W)), torch.float32)
    basis = pkg.TensorBasis(W, D)
    ell = dev(rng.uniform(-1, 1, (B, basis.size())), torch.float32)
    st = pkg.GB300Strategy(torch.float32)
    out = []
    for schedule in (32 | (1 << 16), 256):
        sig = torch.full((B, basis.size()), float("nan"), dtype=torch.float32, device="cuda")
        grad = torch.full((B * L, W), float("nan"), dtype=torch.float32, device="cuda")
        err = pkg.signature(st, None, incr, basis, B, length=L, out=sig, seed=ell, grad=grad, schedule=schedule)
        assert err, err.message
        out.append((host(sig), host(grad)))
    assert np.array_equal(out[0][0], out[1][0]), "signatures differ"
    e = scaled_err(out[0][1], out[1][1])
    assert e <= 2e-6, f"W{W} D{D}: gradients differ by {e:.3e} (scaled)"


@pytest.mark.parametrize("W,D,threads", [(2, 12, 512), (5, 5, 128), (4, 4, 256), (16, 3, 128)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_forward_only_top_level_in_output_row(orc, W, D, threads, dtype):
    """A forward-only call with schedule bit 15 keeps the top level in the
    output row instead of shared memory (as the two-launch form's forward
    launch does): the same arithmetic, so the signatures equal those of the
    shared-memory form bit for bit, and the oracle's within tolerance; ragged,
    with empty and unit paths."""
    rng = np.random.default_rng(W * 71 + D)
    lengths = np.array([0, 1, 5, 17, 2, 9, 0, 12])
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = rng.normal(0, 0.3, (int(offsets[-1]), W))
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(dtype)
    out = []
    for schedule in (threads, threads | (1 << 15)):
        sig = torch.full((len(lengths), basis.size()), float("nan"), dtype=dtype, device="cuda")
        err = pkg.signature(st, None, dev(incr, dtype), basis, len(lengths), offsets=dev(offsets, torch.int64),
                            out=sig, schedule=schedule)
        assert err, err.message
        out.append(host(sig))
    assert np.array_equal(out[0], out[1])
    esig, _ = orc.signature(W, D, incr, offsets)
    assert_close(out[1], esig, TOL_F64 if dtype == torch.float64 else TOL_F32, f"W{W} D{D} top level in the row")


@pytest.mark.parametrize("W,D", [(5, 5), (8, 4)])
def test_fp32_long_paths_within_tolerance(orc, W, D):
    """FP32 forward + reverse on paths of 2048 increments (the longest of the
    uneven-length configuration): the reverse pass recovers each prefix
    through exp(-dx), so its rounding accumulates along the path; signatures
    and gradients stay within 1e-5 of the FP64 oracle (measured about 3e-6
    and 2e-6), for the warp-per-letter kernel and the shared-memory kernel."""
    B, L = 2, 2048
    rng = np.random.default_rng(W * 1000 + L)
    incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    ell = rng.uniform(-1, 1, (B, dim))
    esig, egrad = orc.signature(W, D, incr, np.arange(B + 1) * L, ell=ell)
    st = pkg.GB300Strategy(torch.float32)
    for schedule in (32 | (1 << 16), 256):
        sig = torch.full((B, dim), float("nan"), dtype=torch.float32, device="cuda")
        grad = torch.full((B * L, W), float("nan"), dtype=torch.float32, device="cuda")
        err = pkg.signature(st, None, dev(incr, torch.float32), basis, B, length=L, out=sig,
                            seed=dev(ell, torch.float32), grad=grad, schedule=schedule)
        assert err, err.message
        assert_close(host(sig), esig, TOL_F32, f"W{W} D{D} L{L} schedule {schedule} signature")
        e = scaled_err(host(grad), egrad)
        assert e <= TOL_F32, f"W{W} D{D} L{L} schedule {schedule} gradient: scaled error {e:.3e}"
