"""The allocation-free signature entry point, rpp_gb_signature_static_scratch.

It exists for callers that cannot allocate device memory while they run: a
runtime that owns all device memory through its own allocator and does not
let plugins call cudaMalloc or cudaMallocAsync, a real-time loop that must
not wait on or grow a memory pool, a host that fixes its device-memory budget
up front.  The entry point keeps the only scratch the signature launch needs
(a ragged batch's work counter and longest-first order) in a fixed device
array of the library, so it must give exactly what rpp_gb_signature gives.

These tests call both entry points through the C ABI on the same ragged
batch, twice in a row (the array keeps the previous call's contents, so the
second call checks that each call re-initialises what it reads), on an
equal-length batch, and after the autotuner has recorded a schedule for the
shape (a recorded schedule may ask for two launches, a top level in global
memory or a cotangent workspace; the entry point must honour what needs no
allocation and drop the workspace).  The device's stream-ordered memory pool
(the one cudaMallocAsync draws from) is watched through the driver API: its
used-memory high-water mark must not rise during a call.  The entry point
also refuses what it cannot do without allocating.  This file is named to be
collected last."""
import ctypes
import importlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")

F32, F64 = 0, 1

# CUmemPool_attribute values (cuda.h)
_POOL_USED_MEM_CURRENT = 7
_POOL_USED_MEM_HIGH = 8


class _PoolWatch:
    """The device's default stream-ordered pool, read through libcuda."""

    def __init__(self, device=0):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), device) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def _get(self, attr):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        # setting the high-water mark to zero resets it to the current use
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, _POOL_USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def used(self):
        return self._get(_POOL_USED_MEM_CURRENT)

    def high(self):
        return self._get(_POOL_USED_MEM_HIGH)


def _ragged(rng, B, max_len, W):
    lengths = rng.integers(0, max_len + 1, B)
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    return offsets, rng.normal(0, 0.2, (int(offsets[-1]), W))


def _call(name, plan, incr, offsets, B, sig, seed, grad, dim, length=0):
    lib = pkg.library()
    stream = torch.cuda.current_stream().cuda_stream
    dtype = F64 if incr.dtype == torch.float64 else F32
    rc = getattr(lib, name)(plan, stream, dtype, incr.data_ptr(), None if offsets is None else offsets.data_ptr(),
                            length, B, sig.data_ptr(), dim, seed.data_ptr(), dim, grad.data_ptr())
    msg = lib.rpp_gb_last_error_string()
    return rc, (msg.decode() if msg else "")


def _assert_same(sig, grad, sig_ref, grad_ref, what):
    for got, want, name in ((sig, sig_ref, "signature"), (grad, grad_ref, "gradient")):
        scale = torch.clamp(torch.maximum(got.abs(), want.abs()), min=1.0)
        err = float(((got - want).abs() / scale).max())
        assert err <= 1e-12, f"{what} {name}: relative error {err:.3e}"


def _static_call_without_pool_growth(pool, *args, **kw):
    """One call of the allocation-free entry point; asserts that the pool's
    used memory never rose above its level before the call."""
    torch.cuda.synchronize()
    before = pool.used()
    pool.reset_high()
    rc, msg = _call("rpp_gb_signature_static_scratch", *args, **kw)
    torch.cuda.synchronize()
    assert pool.high() == before, f"stream-ordered pool grew from {before} to {pool.high()} bytes"
    return rc, msg


def test_static_scratch_matches_allocating_entry_on_two_calls():
    W, D, B = 4, 4, 300
    rng = np.random.default_rng(77)
    offsets_h, incr_h = _ragged(rng, B, 64, W)
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    plan = basis.plan(0)
    incr = torch.from_numpy(incr_h).cuda()
    offsets = torch.from_numpy(offsets_h).cuda()
    seed = torch.from_numpy(rng.uniform(-1, 1, (B, dim))).cuda()
    sig_ref = torch.full((B, dim), float("nan"), dtype=torch.float64, device="cuda")
    grad_ref = torch.full_like(incr, float("nan"))
    rc, msg = _call("rpp_gb_signature", plan, incr, offsets, B, sig_ref, seed, grad_ref, dim)
    assert rc == 0, msg
    pool = _PoolWatch()
    for call in range(2):
        sig = torch.full_like(sig_ref, float("nan"))
        grad = torch.full_like(grad_ref, float("nan"))
        rc, msg = _static_call_without_pool_growth(pool, plan, incr, offsets, B, sig, seed, grad, dim)
        assert rc == 0, f"call {call}: {msg}"
        _assert_same(sig, grad, sig_ref, grad_ref, f"call {call}")


def test_static_scratch_equal_length_batch():
    W, D, B, L = 5, 5, 64, 40
    rng = np.random.default_rng(78)
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    plan = basis.plan(0)
    incr = torch.from_numpy(rng.normal(0, 1 / np.sqrt(L), (B * L, W))).cuda()
    seed = torch.from_numpy(rng.uniform(-1, 1, (B, dim))).cuda()
    sig_ref = torch.full((B, dim), float("nan"), dtype=torch.float64, device="cuda")
    grad_ref = torch.full_like(incr, float("nan"))
    rc, msg = _call("rpp_gb_signature", plan, incr, None, B, sig_ref, seed, grad_ref, dim, length=L)
    assert rc == 0, msg
    pool = _PoolWatch()
    sig = torch.full_like(sig_ref, float("nan"))
    grad = torch.full_like(grad_ref, float("nan"))
    rc, msg = _static_call_without_pool_growth(pool, plan, incr, None, B, sig, seed, grad, dim, length=L)
    assert rc == 0, msg
    _assert_same(sig, grad, sig_ref, grad_ref, "equal lengths")


@pytest.mark.parametrize("W,D,B,max_len", [(2, 12, 1024, 48), (5, 5, 1024, 96)])
def test_static_scratch_after_tuning(W, D, B, max_len):
    """The autotuner records a schedule word for the shape; the allocation-free
    entry point must read it as a schedule (CTA size, cap, two launches, top
    level in global memory), not as a thread count, and drop only the
    cotangent workspace."""
    rng = np.random.default_rng(W * 100 + D)
    offsets_h, incr_h = _ragged(rng, B, max_len, W)
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    plan = basis.plan(0)
    lib = pkg.library()
    incr = torch.from_numpy(incr_h).cuda()
    offsets = torch.from_numpy(offsets_h).cuda()
    seed = torch.from_numpy(rng.uniform(-1, 1, (B, dim))).cuda()
    sig_ref = torch.full((B, dim), float("nan"), dtype=torch.float64, device="cuda")
    grad_ref = torch.full_like(incr, float("nan"))
    chosen = ctypes.c_int32(0)
    ms = ctypes.c_float(0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.rpp_gb_signature_tune(plan, stream, F64, incr.data_ptr(), offsets.data_ptr(), 0, B,
                                   sig_ref.data_ptr(), dim, seed.data_ptr(), dim, grad_ref.data_ptr(),
                                   ctypes.byref(chosen), ctypes.byref(ms))
    assert rc == 0, lib.rpp_gb_last_error_string()
    print(f"W{W} D{D}: tuned schedule {chosen.value:#x}")
    rc, msg = _call("rpp_gb_signature", plan, incr, offsets, B, sig_ref, seed, grad_ref, dim)
    assert rc == 0, msg
    pool = _PoolWatch()
    for call in range(2):
        sig = torch.full_like(sig_ref, float("nan"))
        grad = torch.full_like(grad_ref, float("nan"))
        rc, msg = _static_call_without_pool_growth(pool, plan, incr, offsets, B, sig, seed, grad, dim)
        assert rc == 0, f"schedule {chosen.value:#x}, call {call}: {msg}"
        _assert_same(sig, grad, sig_ref, grad_ref, f"schedule {chosen.value:#x}, call {call}")


@pytest.mark.parametrize("W,D", [(5, 5), (8, 4)])
def test_static_scratch_fp32_warp_per_letter_kernel(W, D):
    """FP32 calls of these shapes take the warp-per-letter forward + reverse
    kernel without a recorded schedule; through the allocation-free entry
    point they run the same kernel (results equal bit for bit) and allocate
    nothing."""
    B = 200
    rng = np.random.default_rng(W * 31 + D)
    offsets_h, incr_h = _ragged(rng, B, 40, W)
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    plan = basis.plan(0)
    incr = torch.from_numpy(incr_h).to("cuda", torch.float32)
    offsets = torch.from_numpy(offsets_h).cuda()
    seed = torch.from_numpy(rng.uniform(-1, 1, (B, dim))).to("cuda", torch.float32)
    sig_ref = torch.full((B, dim), float("nan"), dtype=torch.float32, device="cuda")
    grad_ref = torch.full_like(incr, float("nan"))
    rc, msg = _call("rpp_gb_signature", plan, incr, offsets, B, sig_ref, seed, grad_ref, dim)
    assert rc == 0, msg
    pool = _PoolWatch()
    sig = torch.full_like(sig_ref, float("nan"))
    grad = torch.full_like(grad_ref, float("nan"))
    rc, msg = _static_call_without_pool_growth(pool, plan, incr, offsets, B, sig, seed, grad, dim)
    assert rc == 0, msg
    torch.cuda.synchronize()
    assert torch.equal(sig, sig_ref) and torch.equal(grad, grad_ref)


def test_static_scratch_refuses_what_needs_an_allocation():
    lib = pkg.library()
    rng = np.random.default_rng(3)
    offsets_h, incr_h = _ragged(rng, 4, 8, 6)
    incr = torch.from_numpy(incr_h).cuda()
    offsets = torch.from_numpy(offsets_h).cuda()
    # a state that does not fit shared memory (width 6, depth 6, FP64)
    big = pkg.TensorBasis(6, 6)
    dim = big.size()
    sig = torch.empty(4, dim, dtype=torch.float64, device="cuda")
    seed = torch.zeros_like(sig)
    grad = torch.empty_like(incr)
    rc, msg = _call("rpp_gb_signature_static_scratch", big.plan(0), incr, offsets, 4, sig, seed, grad, dim)
    assert rc == int(pkg.ErrorCode.NotImplemented) and "shared memory" in msg
    # a ragged batch beyond the array's capacity is refused before any launch
    small = pkg.TensorBasis(2, 2)
    dim2 = small.size()
    sig2 = torch.empty(1, dim2, dtype=torch.float64, device="cuda")
    rc, msg = _call("rpp_gb_signature_static_scratch", small.plan(0), incr, offsets, 3_000_000, sig2,
                    torch.zeros_like(sig2), torch.empty_like(incr), dim2)
    assert rc == int(pkg.ErrorCode.OutOfBounds) and "capacity" in msg
    assert ctypes.c_int(rc).value != 0
