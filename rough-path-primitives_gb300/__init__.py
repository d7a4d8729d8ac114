"""GB300-native batched free-tensor operations behind RoughPathPrimitives'
operation API.

This module is the Python face of the C ABI in ``include/rpp_gb300.h``; it
mirrors the reference's operation front ends (``rpp::ops::<op>(strategy,
config, batches..., basis, num_batches, scalars...)``, e.g.
include/rpp/operations/basic/ft_mul.hpp:48-79) with the same names, argument
order and meaning, and the same error convention: every operation returns an
``Error`` whose truth value is True on success
(include/rpp/support/error.hpp:140-146).  The reference's C++ callers use the
``GB300Strategy`` header in ``include/rpp/gpu/gb300/strategy.hpp`` instead.

Device memory and streams come from PyTorch tensors (plumbing only); all
arithmetic runs in the sm_103a kernels of ``librpp_gb300.so``.  There is no
host fallback: a missing library raises.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass, field

import numpy as np

from . import _lib

__all__ = [
    "ErrorCode", "Error", "TensorBasis", "LieBasis", "GB300Strategy", "DeviceLaunchConfig",
    "make_tensor_batch", "make_lie_batch", "SparseMatrix", "make_t2l_matrix", "make_l2t_matrix",
    "FTInplaceFMAType", "ft_mul", "ft_fma", "ft_inplace_fma", "ft_inplace_mul", "ft_exp",
    "ft_fmexp", "ft_log", "ft_adj_lmul", "ft_adj_rmul", "tensor_antipode", "tensor_reflect",
    "tensor_generalised_antipode", "vector_assign", "vector_set_constant",
    "tensor_set_identity", "tensor_add_identity", "sparse_matrix_vector_product",
    "tensor_to_lie", "lie_to_tensor", "signature", "signature_backward", "signature_tune", "exp_letter_vjp",
    "signature_host", "SignatureJob", "signature_group",
    "st_mul", "st_fma", "st_inplace_fma", "st_adj_mul", "left_hs_mul", "left_hs_adj_lmul", "left_hs_adj_rmul",
    "tensor_pairing", "make_scalar_batch", "tensor_log_to_lie", "lie_to_tensor_exp", "build", "library",
]


def build(jobs: int = 8) -> None:
    """Compile librpp_gb300.so for sm_103a."""
    _lib.build(jobs)


def library():
    """The loaded ctypes library (raises if it was not built)."""
    return _lib.load()


class ErrorCode(enum.IntEnum):
    """rpp::ErrorCode (include/rpp/support/error.hpp:28-39)."""

    Success = 0
    Cancelled = 1
    Unknown = 2
    InvalidArgument = 3
    Timeout = 4
    OutOfResources = 5
    ContractViolation = 6
    OutOfBounds = 7
    NotImplemented = 8
    Internal = 9


@dataclass
class Error:
    """rpp::Error<char const*>: truthy on success."""

    code: ErrorCode
    message: str = ""

    def __bool__(self) -> bool:
        return self.code == ErrorCode.Success

    def raise_if_failed(self) -> "Error":
        if not self:
            raise RuntimeError(f"{self.code.name}: {self.message}")
        return self


def _status(rc: int) -> Error:
    if rc == 0:
        return Error(ErrorCode.Success)
    msg = _lib.load().rpp_gb_last_error_string()
    return Error(ErrorCode(rc), msg.decode() if msg else "")


def _torch():
    import torch

    return torch


_F32, _F64 = 0, 1


class TensorBasis:
    """Tensor basis of width W and depth D (include/rpp/basis/tensor_basis.hpp):
    degree_begin[n] = (W^n - 1)/(W - 1).  Holds one device plan per CUDA device,
    created on first use (the plan caches what the reference re-uploads on
    every launch)."""

    def __init__(self, width: int, depth: int):
        self.width, self.depth = int(width), int(depth)
        db, p = [0], 1
        for _ in range(self.depth + 1):
            db.append(db[-1] + p)
            p *= self.width
        self.degree_begin = db
        self._plans: dict[int, int] = {}

    def size(self) -> int:
        return self.degree_begin[self.depth + 1]

    def start_of_degree(self, d: int) -> int:
        return self.degree_begin[d]

    def end_of_degree(self, d: int) -> int:
        return self.degree_begin[d + 1]

    def size_of_degree(self, d: int) -> int:
        return self.degree_begin[d + 1] - self.degree_begin[d]

    def truncate(self, depth: int) -> "TensorBasis":
        return TensorBasis(self.width, min(self.depth, depth))

    def plan(self, device: int) -> int:
        h = self._plans.get(device)
        if h is None:
            lib = _lib.load()
            out = ctypes.c_void_p()
            rc = lib.rpp_gb_plan_create(ctypes.byref(out), self.width, self.depth, device)
            _status(rc).raise_if_failed()
            h = out.value
            self._plans[device] = h
        return h

    def __del__(self):
        try:
            lib = _lib.load()
            for h in self._plans.values():
                lib.rpp_gb_plan_destroy(h)
        except Exception:  # interpreter shutdown
            pass


class LieBasis:
    """Hall basis (include/rpp/basis/hall_basis.hpp, lie_basis.hpp): key 0 is a
    sentinel, keys 1..W the letters; ``true_size`` slots are stored."""

    def __init__(self, width: int, depth: int):
        self.width, self.depth = int(width), int(depth)
        lib = _lib.load()
        ts = ctypes.c_int64()
        _status(lib.rpp_gb_lie_basis(self.width, self.depth, ctypes.byref(ts), None, None)).raise_if_failed()
        self._true_size = ts.value
        db = np.zeros(self.depth + 2, np.int64)
        pairs = np.zeros(2 * ts.value, np.int64)
        _status(lib.rpp_gb_lie_basis(self.width, self.depth, None, _i64p(db), _i64p(pairs))).raise_if_failed()
        self.degree_begin = db.tolist()
        self.pairs = pairs.reshape(-1, 2)

    def true_size(self) -> int:
        return self._true_size

    def size(self) -> int:
        return 0 if self.width <= 1 or self.depth == 0 else self._true_size - 1

    def start_of_degree(self, d: int) -> int:
        return self.degree_begin[d]

    def end_of_degree(self, d: int) -> int:
        return self.degree_begin[d + 1]


def _i64p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


@dataclass
class TensorBatch:
    """Batch of dense tensor views (include/rpp/views/dense_tensor_view.hpp:
    make_tensor_batch): element b is the tensor whose coefficient 0 sits at
    element ``offset + b*stride`` of ``data``.  Only coefficients inside the
    degree range are ever touched, so ``offset`` may point before the buffer
    (e.g. ``-1`` views a row of increments as the degree-1 part of a tensor)."""

    data: object
    stride: int
    min_degree: int
    max_degree: int
    offset: int = 0

    def arg(self) -> _lib.TensorArg:
        ptr = self.data.data_ptr() + self.offset * self.data.element_size()
        return _lib.TensorArg(ptr, self.stride, self.min_degree, self.max_degree)

    def truncate(self, lo: int, hi: int) -> "TensorBatch":
        return TensorBatch(self.data, self.stride, max(lo, self.min_degree), min(hi, self.max_degree), self.offset)


@dataclass
class LieBatch:
    """Batch of Lie-vector views (include/rpp/views/dense_lie_view.hpp)."""

    data: object
    stride: int
    min_degree: int
    max_degree: int


def make_tensor_batch(data, stride: int, min_degree: int, max_degree: int, offset: int = 0) -> TensorBatch:
    return TensorBatch(data, int(stride), int(min_degree), int(max_degree), int(offset))


def make_lie_batch(data, stride: int, min_degree: int, max_degree: int) -> LieBatch:
    return LieBatch(data, int(stride), int(min_degree), int(max_degree))


@dataclass
class GB300Strategy:
    """The new ``gpu`` strategy: Accum is the scalar/accumulation dtype
    (torch.float32 or torch.float64), device the CUDA ordinal."""

    accum: object = None
    device: int = 0

    def dtype_code(self) -> int:
        torch = _torch()
        acc = self.accum if self.accum is not None else torch.float64
        if acc == torch.float64:
            return _F64
        if acc == torch.float32:
            return _F32
        raise ValueError("GB300Strategy supports float32 and float64")

    def torch_dtype(self):
        torch = _torch()
        return self.accum if self.accum is not None else torch.float64


@dataclass
class DeviceLaunchConfig:
    """gpu::DeviceLaunchConfig (include/rpp/gpu/device.hpp:21-24): the stream
    (a torch.cuda.Stream, a raw cudaStream_t int, or None for torch's current
    stream).  Launch attributes are accepted for interface parity."""

    stream: object = None
    launch_attributes: list = field(default_factory=list)

    def handle(self, device: int) -> int:
        s = self.stream
        if s is None:
            torch = _torch()
            return torch.cuda.current_stream(device).cuda_stream
        if isinstance(s, int):
            return s
        return s.cuda_stream


class FTInplaceFMAType(enum.IntEnum):
    """include/rpp/operations/basic/ft_inplace_fma.hpp:17-21"""

    AEqualsBCPlusA = 0
    AEqualsABPlusC = 1
    AEqualsBAPlusC = 2


def _check_batches(strategy: GB300Strategy, *batches):
    dt = strategy.torch_dtype()
    for b in batches:
        if b is None:
            continue
        t = b.data
        if not getattr(t, "is_cuda", False):
            raise ValueError("batch data must be a CUDA tensor (the GB300 strategy has no host path)")
        if t.dtype != dt:
            raise ValueError(f"batch dtype {t.dtype} does not match the strategy's {dt}")


def _p(b):
    return None if b is None else ctypes.byref(b.arg())


def _cfg(config):
    return config if config is not None else DeviceLaunchConfig()


# --------------------------------------------------------------------------
# Operations.  Each follows the argument order of its reference front end.
# --------------------------------------------------------------------------

def ft_mul(strategy, config, out, lhs, rhs, basis, num_batches, beta=1.0) -> Error:
    """include/rpp/operations/basic/ft_mul.hpp:53-79"""
    _check_batches(strategy, out, lhs, rhs)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_mul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                     strategy.dtype_code(), _p(out), _p(lhs), _p(rhs), num_batches, beta))


def ft_fma(strategy, config, out, a, b, c, basis, num_batches, alpha=1.0, beta=1.0) -> Error:
    """include/rpp/operations/basic/ft_fma.hpp:54-83"""
    _check_batches(strategy, out, a, b, c)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_fma(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                     strategy.dtype_code(), _p(out), _p(a), _p(b), _p(c), num_batches,
                                     alpha, beta))


def ft_inplace_fma(fma_type, strategy, config, a, b, c, basis, num_batches, alpha=1.0, beta=1.0) -> Error:
    """include/rpp/operations/basic/ft_inplace_fma.hpp:64-96"""
    _check_batches(strategy, a, b, c)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_inplace_fma(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                             strategy.dtype_code(), int(fma_type), _p(a), _p(b), _p(c),
                                             num_batches, alpha, beta))


def ft_inplace_mul(strategy, config, lhs, rhs, basis, num_batches, beta=1.0) -> Error:
    """include/rpp/operations/basic/ft_inplace_mul.hpp:40-69"""
    _check_batches(strategy, lhs, rhs)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_inplace_mul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                             strategy.dtype_code(), _p(lhs), _p(rhs), num_batches, beta))


def ft_exp(strategy, config, out, arg, basis, num_batches) -> Error:
    """include/rpp/operations/intermediate/ft_exp.hpp:84-112"""
    _check_batches(strategy, out, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_exp(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                     strategy.dtype_code(), _p(out), _p(arg), num_batches))


def ft_fmexp(strategy, config, out, multiplier, exponent, basis, num_batches) -> Error:
    """include/rpp/operations/intermediate/ft_fmexp.hpp:91-121"""
    _check_batches(strategy, out, multiplier, exponent)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_fmexp(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                       strategy.dtype_code(), _p(out), _p(multiplier), _p(exponent),
                                       num_batches))


def ft_log(strategy, config, out, arg, basis, num_batches) -> Error:
    """include/rpp/operations/intermediate/ft_log.hpp:87-114"""
    _check_batches(strategy, out, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_log(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                     strategy.dtype_code(), _p(out), _p(arg), num_batches))


def ft_adj_lmul(strategy, config, out, op, arg, basis, num_batches) -> Error:
    """include/rpp/operations/basic/ft_adj_lmul.hpp:44-73"""
    _check_batches(strategy, out, op, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_adj_lmul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                          strategy.dtype_code(), _p(out), _p(op), _p(arg), num_batches))


def ft_adj_rmul(strategy, config, out, op, arg, basis, num_batches) -> Error:
    """include/rpp/operations/basic/ft_adj_rmul.hpp:42-71"""
    _check_batches(strategy, out, op, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_ft_adj_rmul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                          strategy.dtype_code(), _p(out), _p(op), _p(arg), num_batches))


# --------------------------------------------------------------------------
# Shuffle algebra and the tensor pairing.
# --------------------------------------------------------------------------

def st_mul(strategy, config, out, lhs, rhs, basis, num_batches, beta=1.0) -> Error:
    """include/rpp/operations/basic/st_mul.hpp:53-79: out = beta * lhs sh rhs."""
    _check_batches(strategy, out, lhs, rhs)
    lib = _lib.load()
    return _status(lib.rpp_gb_st_mul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                     strategy.dtype_code(), _p(out), _p(lhs), _p(rhs), num_batches, beta))


def st_fma(strategy, config, out, a, b, c, basis, num_batches, alpha=1.0, beta=1.0) -> Error:
    """include/rpp/operations/basic/st_fma.hpp:56-85: out = alpha*a + beta * b sh c."""
    _check_batches(strategy, out, a, b, c)
    lib = _lib.load()
    return _status(lib.rpp_gb_st_fma(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                     strategy.dtype_code(), _p(out), _p(a), _p(b), _p(c), num_batches,
                                     alpha, beta))


def st_inplace_fma(strategy, config, a, b, c, basis, num_batches, alpha=1.0, beta=1.0) -> Error:
    """include/rpp/operations/basic/st_inplace_fma.hpp:50-80: a = alpha*a + beta * b sh c."""
    _check_batches(strategy, a, b, c)
    lib = _lib.load()
    return _status(lib.rpp_gb_st_inplace_fma(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                             strategy.dtype_code(), _p(a), _p(b), _p(c), num_batches, alpha, beta))


def st_adj_mul(strategy, config, out, op, arg, basis, num_batches) -> Error:
    """include/rpp/operations/basic/st_adj_mul.hpp:46-69: the adjoint of x -> op sh x."""
    _check_batches(strategy, out, op, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_st_adj_mul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                         strategy.dtype_code(), _p(out), _p(op), _p(arg), num_batches))


def left_hs_mul(strategy, config, out, integrator, integrand, basis, num_batches, beta=1.0) -> Error:
    """include/rpp/operations/basic/left_hs_mul.hpp:59-87: out = beta * integrator < integrand."""
    _check_batches(strategy, out, integrator, integrand)
    lib = _lib.load()
    return _status(lib.rpp_gb_left_hs_mul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                          strategy.dtype_code(), _p(out), _p(integrator), _p(integrand),
                                          num_batches, beta))


def left_hs_adj_lmul(strategy, config, out, op, arg, basis, num_batches, beta=1.0) -> Error:
    """include/rpp/operations/basic/left_hs_adj_lmul.hpp:39-57: adjoint of
    y -> op < y (op = the fixed integrator, arg = the cotangent)."""
    _check_batches(strategy, out, op, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_left_hs_adj_lmul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                               strategy.dtype_code(), _p(out), _p(op), _p(arg), num_batches, beta))


def left_hs_adj_rmul(strategy, config, out, op, arg, basis, num_batches, beta=1.0) -> Error:
    """include/rpp/operations/basic/left_hs_adj_rmul.hpp:39-57: adjoint of
    x -> x < arg (op = the cotangent, arg = the fixed integrand)."""
    _check_batches(strategy, out, op, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_left_hs_adj_rmul(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                               strategy.dtype_code(), _p(out), _p(op), _p(arg), num_batches, beta))


class ScalarBatch:
    """rpp::make_scalar_batch (include/rpp/views/scalar_view.hpp:53-60): one
    scalar per batch element, contiguous."""

    def __init__(self, data):
        self.data = data


def make_scalar_batch(data) -> ScalarBatch:
    return ScalarBatch(data)


def tensor_pairing(strategy, config, result, functional, arg, basis, num_batches) -> Error:
    """include/rpp/operations/basic/tensor_pairing.hpp:47-73: result[b] =
    <functional_b, arg_b> over the degrees both views hold."""
    _check_batches(strategy, result, functional, arg)
    t = result.data
    if t.dim() != 1 or not t.is_contiguous() or t.numel() < num_batches:
        raise ValueError("tensor_pairing: result must be a contiguous 1-D tensor of num_batches scalars")
    lib = _lib.load()
    return _status(lib.rpp_gb_tensor_pairing(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                             strategy.dtype_code(), t.data_ptr(), _p(functional), _p(arg),
                                             num_batches))


def tensor_generalised_antipode(policy, strategy, config, out, arg, basis, num_batches) -> Error:
    """include/rpp/operations/basic/tensor_generalised_antipode.hpp:42-69;
    policy 1 = SignByDegree, 0 = NoSigning."""
    _check_batches(strategy, out, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_tensor_antipode(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                              strategy.dtype_code(), int(policy), _p(out), _p(arg),
                                              num_batches))


def tensor_antipode(strategy, config, out, arg, basis, num_batches) -> Error:
    """include/rpp/operations/basic/tensor_antipode.hpp"""
    return tensor_generalised_antipode(1, strategy, config, out, arg, basis, num_batches)


def tensor_reflect(strategy, config, out, arg, basis, num_batches) -> Error:
    """include/rpp/operations/basic/tensor_reflect.hpp"""
    return tensor_generalised_antipode(0, strategy, config, out, arg, basis, num_batches)


def vector_assign(strategy, config, out, arg, basis, num_batches) -> Error:
    _check_batches(strategy, out, arg)
    lib = _lib.load()
    return _status(lib.rpp_gb_vector_assign(basis.plan(strategy.device), _cfg(config).handle(strategy.device),
                                            strategy.dtype_code(), _p(out), _p(arg), num_batches))


def vector_set_constant(strategy, config, out, basis, num_batches, value) -> Error:
    _check_batches(strategy, out)
    lib = _lib.load()
    return _status(lib.rpp_gb_vector_set_constant(basis.plan(strategy.device),
                                                  _cfg(config).handle(strategy.device), strategy.dtype_code(),
                                                  _p(out), num_batches, value))


def tensor_set_identity(strategy, config, out, basis, num_batches, scalar=1.0) -> Error:
    _check_batches(strategy, out)
    lib = _lib.load()
    return _status(lib.rpp_gb_tensor_set_identity(basis.plan(strategy.device),
                                                  _cfg(config).handle(strategy.device), strategy.dtype_code(),
                                                  _p(out), num_batches, scalar))


def tensor_add_identity(strategy, config, out, basis, num_batches, scalar=1.0) -> Error:
    _check_batches(strategy, out)
    lib = _lib.load()
    return _status(lib.rpp_gb_tensor_add_identity(basis.plan(strategy.device),
                                                  _cfg(config).handle(strategy.device), strategy.dtype_code(),
                                                  _p(out), num_batches, scalar))


# --------------------------------------------------------------------------
# Sparse matrices and the Lie <-> tensor conversions.
# --------------------------------------------------------------------------

class SparseMatrix:
    """A compressed matrix uploaded once (include/rpp/sparse/detail/
    compressed_matrix.hpp).  ``fmt`` is "csr" or "csc"; outer_dim counts rows
    (CSR) or columns (CSC).  Host arrays are kept for inspection."""

    def __init__(self, fmt, offsets, indices, values, outer_dim, inner_dim, device=0):
        self.format = fmt
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self.indices = np.ascontiguousarray(indices, dtype=np.int64)
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        self.outer_dim, self.inner_dim = int(outer_dim), int(inner_dim)
        self.rows = self.outer_dim if fmt == "csr" else self.inner_dim
        self.cols = self.inner_dim if fmt == "csr" else self.outer_dim
        self._handles: dict[int, int] = {}
        self._default_device = device

    def nnz(self) -> int:
        return int(self.indices.size)

    def handle(self, device: int) -> int:
        h = self._handles.get(device)
        if h is None:
            lib = _lib.load()
            out = ctypes.c_void_p()
            rc = lib.rpp_gb_matrix_create(
                ctypes.byref(out), 0 if self.format == "csr" else 1, self.outer_dim, self.inner_dim, self.nnz(),
                _i64p(self.offsets), _i64p(self.indices),
                self.values.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), device)
            _status(rc).raise_if_failed()
            h = out.value
            self._handles[device] = h
        return h

    def __del__(self):
        try:
            lib = _lib.load()
            for h in self._handles.values():
                lib.rpp_gb_matrix_destroy(h)
        except Exception:
            pass


def _conversion(lie_basis: LieBasis, which: int) -> SparseMatrix:
    lib = _lib.load()
    outer, inner, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    _status(lib.rpp_gb_conversion_matrix(lie_basis.width, lie_basis.depth, which, ctypes.byref(outer),
                                         ctypes.byref(inner), ctypes.byref(nnz), None, None, None)).raise_if_failed()
    off = np.zeros(outer.value + 1 if which == 0 else max(outer.value, lie_basis.true_size() - 1) + 1, np.int64)
    idx = np.zeros(nnz.value, np.int64)
    val = np.zeros(nnz.value, np.float64)
    _status(lib.rpp_gb_conversion_matrix(lie_basis.width, lie_basis.depth, which, None, None, None, _i64p(off),
                                         _i64p(idx), val.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
                                         )).raise_if_failed()
    return SparseMatrix("csc", off[: outer.value + 1], idx, val, outer.value, inner.value)


def make_t2l_matrix(lie_basis: LieBasis) -> SparseMatrix:
    """include/rpp/sparse/t2l_matrix.hpp:57-142 (CSC, rows = Lie index key-1,
    columns = tensor index)."""
    return _conversion(lie_basis, 0)


def make_l2t_matrix(lie_basis: LieBasis) -> SparseMatrix:
    """include/rpp/sparse/l2t_matrix.hpp:58-114 (CSC, rows = tensor index,
    columns = Lie index key-1)."""
    return _conversion(lie_basis, 1)


def _vec(batch, basis) -> _lib.VectorArg:
    begin = basis.degree_begin[batch.min_degree]
    end = basis.degree_begin[min(batch.max_degree, basis.depth) + 1]
    return _lib.VectorArg(batch.data.data_ptr(), batch.stride, begin, max(0, end - begin))


def sparse_matrix_vector_product(strategy, config, out, arg, out_basis, arg_basis, num_batches, matrix,
                                 alpha=1.0) -> Error:
    """include/rpp/operations/linalg/sparse_matrix_vector.hpp:63-96 with the
    CPU strategy's begin-relative indexing."""
    _check_batches(strategy, out, arg)
    lib = _lib.load()
    o, a = _vec(out, out_basis), _vec(arg, arg_basis)
    return _status(lib.rpp_gb_sparse_matrix_vector(matrix.handle(strategy.device),
                                                   _cfg(config).handle(strategy.device), strategy.dtype_code(),
                                                   ctypes.byref(o), ctypes.byref(a), num_batches, alpha))


def tensor_to_lie(strategy, config, out, arg, lie_basis, tensor_basis, num_batches, matrix) -> Error:
    """include/rpp/operations/basic/tensor_to_lie.hpp:71-103"""
    return sparse_matrix_vector_product(strategy, config, out, arg, lie_basis, tensor_basis, num_batches, matrix)


def lie_to_tensor(strategy, config, out, arg, tensor_basis, lie_basis, num_batches, matrix) -> Error:
    """include/rpp/operations/basic/lie_to_tensor.hpp:76-108"""
    return sparse_matrix_vector_product(strategy, config, out, arg, tensor_basis, lie_basis, num_batches, matrix)


def tensor_log_to_lie(strategy, config, out, arg, lie_basis, tensor_basis, num_batches, matrix,
                      log_degrees=None, alpha=1.0) -> Error:
    """Fused ft_log + tensor_to_lie (rpp_gb_log_to_lie): out (a Lie batch) =
    alpha * M * log(arg) on the tensor view ``log_degrees`` (default: every
    degree), without writing the log tensor."""
    _check_batches(strategy, out, arg)
    lo, hi = log_degrees if log_degrees is not None else (0, tensor_basis.depth)
    lib = _lib.load()
    o = _vec(out, lie_basis)
    return _status(lib.rpp_gb_log_to_lie(tensor_basis.plan(strategy.device), matrix.handle(strategy.device),
                                         _cfg(config).handle(strategy.device), strategy.dtype_code(),
                                         ctypes.byref(o), _p(arg), int(lo), int(hi), num_batches, alpha))


def lie_to_tensor_exp(strategy, config, out, multiplier, arg, tensor_basis, lie_basis, num_batches, matrix,
                      tensor_degrees=None, alpha=1.0) -> Error:
    """Fused lie_to_tensor + ft_exp / ft_fmexp (rpp_gb_lie_to_tensor_exp):
    X = alpha * M * arg on the tensor view ``tensor_degrees`` (default: every
    degree) of a zero tensor, out = exp(X) or multiplier (x) exp(X)."""
    _check_batches(strategy, out, multiplier, arg)
    lo, hi = tensor_degrees if tensor_degrees is not None else (0, tensor_basis.depth)
    lib = _lib.load()
    a = _vec(arg, lie_basis)
    return _status(lib.rpp_gb_lie_to_tensor_exp(tensor_basis.plan(strategy.device), matrix.handle(strategy.device),
                                                _cfg(config).handle(strategy.device), strategy.dtype_code(), _p(out),
                                                _p(multiplier), ctypes.byref(a), int(lo), int(hi), num_batches,
                                                alpha))


# --------------------------------------------------------------------------
# Signatures (new fused entry points).
# --------------------------------------------------------------------------

def _ptr(t):
    return None if t is None else t.data_ptr()


def signature(strategy, config, increments, basis, num_batches, *, length=None, offsets=None, out=None,
              out_stride=None, seed=None, seed_stride=None, grad=None, schedule=None) -> Error:
    """Signatures of piecewise-linear paths in one launch (rpp_gb_signature).

    ``increments``: CUDA tensor [total_steps, width]; path b owns rows
    offsets[b]..offsets[b+1] (``offsets``: CUDA int64 [num_batches + 1]) or,
    without offsets, rows b*length..(b+1)*length.  ``out`` receives S(x_b) at
    stride ``out_stride`` (default: the tensor dimension).  With ``seed`` and
    ``grad`` the launch also writes d/dx sum_b <seed_b, S(x_b)> into ``grad``
    (same layout as ``increments``)."""
    _check_batches(strategy, *(TensorBatch(t, 0, 0, 0) for t in (increments, out, seed, grad) if t is not None))
    dim = basis.size()
    lib = _lib.load()
    args = (basis.plan(strategy.device), _cfg(config).handle(strategy.device), strategy.dtype_code(),
            _ptr(increments), _ptr(offsets), 0 if length is None else int(length), num_batches, _ptr(out),
            dim if out_stride is None else out_stride, _ptr(seed), dim if seed_stride is None else seed_stride,
            _ptr(grad))
    if schedule is not None:  # an explicit schedule (rpp_gb_signature_with_schedule)
        return _status(lib.rpp_gb_signature_with_schedule(*args, int(schedule)))
    return _status(lib.rpp_gb_signature(*args))


class SignatureJob:
    """One job of ``signature_group``: the arguments of one ``signature`` call
    (its strategy -- hence dtype --, basis, increments with ``length`` or
    ``offsets``, outputs) and ``threads``, the threads that run one of its
    paths (0: the shape's tuned CTA size, else a heuristic), with bit 26 for
    an FP64 forward + reverse job whose cotangent arrays go to a global
    workspace."""

    def __init__(self, strategy, increments, basis, num_batches, *, length=None, offsets=None, out=None,
                 out_stride=None, seed=None, seed_stride=None, grad=None, threads=0):
        _check_batches(strategy, *(TensorBatch(t, 0, 0, 0) for t in (increments, out, seed, grad) if t is not None))
        self.strategy, self.basis = strategy, basis
        self.tensors = (increments, offsets, out, seed, grad)  # kept alive with the job
        dim = basis.size()
        self.arg = _lib.SignatureJobArg(
            basis.plan(strategy.device), strategy.dtype_code(), int(threads), _ptr(increments), _ptr(offsets),
            0 if length is None else int(length), num_batches, _ptr(out), dim if out_stride is None else out_stride,
            _ptr(seed), dim if seed_stride is None else seed_stride, _ptr(grad))


def signature_group(config, jobs, *, schedule=0) -> Error:
    """Several ``signature`` calls -- different (width, depth) shapes and
    precisions -- in one persistent launch (rpp_gb_signature_group).  ``jobs``:
    a sequence of ``SignatureJob`` (1 to 8, one device).  Each job's outputs
    equal those of its own ``signature`` call with ``schedule=job threads``.
    ``schedule``: threads per CTA (bits 0-9, at most 640; 0: 640) and bit 27
    for the D-barrier reverse step."""
    jobs = list(jobs)
    if not jobs:
        raise ValueError("signature_group needs at least one job")
    device = jobs[0].strategy.device
    arr = (_lib.SignatureJobArg * len(jobs))(*(j.arg for j in jobs))
    lib = _lib.load()
    return _status(lib.rpp_gb_signature_group(_cfg(config).handle(device), arr, len(jobs), int(schedule)))


def signature_host(strategy, config, increments, basis, num_batches, *, length, out=None, out_stride=None,
                   seed=None, seed_stride=None, grad=None, chunk=0) -> Error:
    """Signatures of equal-length paths from HOST tensors (rpp_gb_signature_host):
    ``increments`` [num_batches * length, width], ``out``, ``seed`` and ``grad``
    are CPU tensors (pinned, for the copies to overlap the kernels) with the
    layouts of ``signature``.  The batch runs in chunks of ``chunk`` paths
    (0: two) on two internal streams; ``out`` and ``grad`` are complete once
    the configuration's stream has been synchronised."""
    dt = strategy.torch_dtype()
    for t in (increments, out, seed, grad):
        if t is None:
            continue
        if getattr(t, "is_cuda", True):
            raise ValueError("signature_host takes host (CPU) tensors")
        if t.dtype != dt or not t.is_contiguous():
            raise ValueError(f"host tensors must be contiguous {dt}")
    dim = basis.size()
    lib = _lib.load()
    return _status(lib.rpp_gb_signature_host(
        basis.plan(strategy.device), _cfg(config).handle(strategy.device), strategy.dtype_code(),
        _ptr(increments), int(length), num_batches, _ptr(out), dim if out_stride is None else out_stride,
        _ptr(seed), dim if seed_stride is None else seed_stride, _ptr(grad), int(chunk)))


def exp_letter_vjp(strategy, config, cotangent, x, dx, basis, num_batches, *, cotangent_stride=None,
                   x_stride=None, dx_stride=None, x_offset=0, dx_offset=0) -> Error:
    """dx_a = sum_w H[w] d exp(x)[w] / dx_a for degree-one x (rpp_gb_exp_letter_vjp):
    the last link of the stored-prefix reverse pass built from the per-op kernels."""
    _check_batches(strategy, *(TensorBatch(t, 0, 0, 0) for t in (cotangent, x, dx)))
    lib = _lib.load()
    es = x.element_size()
    return _status(lib.rpp_gb_exp_letter_vjp(
        basis.plan(strategy.device), _cfg(config).handle(strategy.device), strategy.dtype_code(),
        cotangent.data_ptr(), basis.size() if cotangent_stride is None else cotangent_stride,
        x.data_ptr() + x_offset * es, basis.width if x_stride is None else x_stride,
        dx.data_ptr() + dx_offset * es, basis.width if dx_stride is None else dx_stride, num_batches))


def signature_tune(strategy, config, increments, basis, num_batches, *, length=None, offsets=None, out=None,
                   out_stride=None, seed=None, seed_stride=None, grad=None):
    """Autotune the signature schedule on these inputs (rpp_gb_signature_tune);
    returns (Error, threads per CTA chosen, ms per launch).  Later ``signature``
    calls of the same shape use the choice."""
    _check_batches(strategy, *(TensorBatch(t, 0, 0, 0) for t in (increments, out, seed, grad) if t is not None))
    dim = basis.size()
    lib = _lib.load()
    threads, ms = ctypes.c_int32(0), ctypes.c_float(0)
    err = _status(lib.rpp_gb_signature_tune(
        basis.plan(strategy.device), _cfg(config).handle(strategy.device), strategy.dtype_code(),
        _ptr(increments), _ptr(offsets), 0 if length is None else int(length), num_batches, _ptr(out),
        dim if out_stride is None else out_stride, _ptr(seed), dim if seed_stride is None else seed_stride,
        _ptr(grad), ctypes.byref(threads), ctypes.byref(ms)))
    return err, threads.value, ms.value


def signature_backward(strategy, config, increments, basis, num_batches, sig, seed, grad, *, length=None,
                       offsets=None, sig_stride=None, seed_stride=None) -> Error:
    """Reverse pass alone from final signatures (rpp_gb_signature_backward)."""
    _check_batches(strategy, *(TensorBatch(t, 0, 0, 0) for t in (increments, sig, seed, grad)))
    dim = basis.size()
    lib = _lib.load()
    return _status(lib.rpp_gb_signature_backward(
        basis.plan(strategy.device), _cfg(config).handle(strategy.device), strategy.dtype_code(),
        _ptr(increments), _ptr(offsets), 0 if length is None else int(length), num_batches, _ptr(sig),
        dim if sig_stride is None else sig_stride, _ptr(seed), dim if seed_stride is None else seed_stride,
        _ptr(grad)))
