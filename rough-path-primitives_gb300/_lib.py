"""ctypes bindings of librpp_gb300.so (the C ABI declared in include/rpp_gb300.h).

The library is built in-tree by ``make -C rough-path-primitives_gb300`` into
``_build/librpp_gb300.so``.  There is no fallback: if the shared library is
missing, ``load()`` raises instead of computing anything on the host.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "librpp_gb300.so")

_lock = threading.Lock()
_lib = None


class TensorArg(ctypes.Structure):
    """rpp_gb_tensor_arg: {data, stride, min_degree, max_degree}."""

    _fields_ = [
        ("data", ctypes.c_void_p),
        ("stride", ctypes.c_int64),
        ("min_degree", ctypes.c_int32),
        ("max_degree", ctypes.c_int32),
    ]


class SignatureJobArg(ctypes.Structure):
    """rpp_gb_signature_job: one job of rpp_gb_signature_group."""

    _fields_ = [
        ("plan", ctypes.c_void_p),
        ("dtype", ctypes.c_int32),
        ("threads", ctypes.c_int32),
        ("incr", ctypes.c_void_p),
        ("offsets", ctypes.c_void_p),
        ("length", ctypes.c_int64),
        ("batch", ctypes.c_int64),
        ("sig", ctypes.c_void_p),
        ("sig_stride", ctypes.c_int64),
        ("seed", ctypes.c_void_p),
        ("seed_stride", ctypes.c_int64),
        ("grad", ctypes.c_void_p),
    ]


class VectorArg(ctypes.Structure):
    """rpp_gb_vector_arg: {data, stride, begin, size}."""

    _fields_ = [
        ("data", ctypes.c_void_p),
        ("stride", ctypes.c_int64),
        ("begin", ctypes.c_int64),
        ("size", ctypes.c_int64),
    ]


# Every exported symbol with its argument types (all return int unless noted).
_P = ctypes.POINTER(TensorArg)
_V = ctypes.POINTER(VectorArg)
_vp, _i32, _i64, _dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
_I64P = ctypes.POINTER(ctypes.c_int64)
_DBLP = ctypes.POINTER(ctypes.c_double)

SIGNATURES = {
    "rpp_gb_plan_create": [ctypes.POINTER(_vp), _i32, _i32, _i32],
    "rpp_gb_plan_destroy": [_vp],
    "rpp_gb_plan_fault": [_vp, ctypes.POINTER(ctypes.c_uint32)],
    "rpp_gb_selftest_bounded_wait": [_vp, _vp],
    "rpp_gb_last_error_string": [],
    "rpp_gb_version": [],
    "rpp_gb_ft_mul": [_vp, _vp, _i32, _P, _P, _P, _i64, _dbl],
    "rpp_gb_ft_fma": [_vp, _vp, _i32, _P, _P, _P, _P, _i64, _dbl, _dbl],
    "rpp_gb_ft_inplace_fma": [_vp, _vp, _i32, _i32, _P, _P, _P, _i64, _dbl, _dbl],
    "rpp_gb_ft_inplace_mul": [_vp, _vp, _i32, _P, _P, _i64, _dbl],
    "rpp_gb_ft_exp": [_vp, _vp, _i32, _P, _P, _i64],
    "rpp_gb_ft_fmexp": [_vp, _vp, _i32, _P, _P, _P, _i64],
    "rpp_gb_ft_log": [_vp, _vp, _i32, _P, _P, _i64],
    "rpp_gb_ft_adj_lmul": [_vp, _vp, _i32, _P, _P, _P, _i64],
    "rpp_gb_ft_adj_rmul": [_vp, _vp, _i32, _P, _P, _P, _i64],
    "rpp_gb_tensor_antipode": [_vp, _vp, _i32, _i32, _P, _P, _i64],
    "rpp_gb_st_mul": [_vp, _vp, _i32, _P, _P, _P, _i64, _dbl],
    "rpp_gb_st_fma": [_vp, _vp, _i32, _P, _P, _P, _P, _i64, _dbl, _dbl],
    "rpp_gb_st_inplace_fma": [_vp, _vp, _i32, _P, _P, _P, _i64, _dbl, _dbl],
    "rpp_gb_st_adj_mul": [_vp, _vp, _i32, _P, _P, _P, _i64],
    "rpp_gb_left_hs_mul": [_vp, _vp, _i32, _P, _P, _P, _i64, _dbl],
    "rpp_gb_left_hs_adj_lmul": [_vp, _vp, _i32, _P, _P, _P, _i64, _dbl],
    "rpp_gb_left_hs_adj_rmul": [_vp, _vp, _i32, _P, _P, _P, _i64, _dbl],
    "rpp_gb_tensor_pairing": [_vp, _vp, _i32, _vp, _P, _P, _i64],
    "rpp_gb_vector_assign": [_vp, _vp, _i32, _P, _P, _i64],
    "rpp_gb_vector_set_constant": [_vp, _vp, _i32, _P, _i64, _dbl],
    "rpp_gb_tensor_set_identity": [_vp, _vp, _i32, _P, _i64, _dbl],
    "rpp_gb_tensor_add_identity": [_vp, _vp, _i32, _P, _i64, _dbl],
    "rpp_gb_matrix_create": [ctypes.POINTER(_vp), _i32, _i64, _i64, _i64, _I64P, _I64P, _DBLP, _i32],
    "rpp_gb_matrix_destroy": [_vp],
    "rpp_gb_matrix_fault": [_vp, ctypes.POINTER(ctypes.c_uint32)],
    "rpp_gb_sparse_matrix_vector": [_vp, _vp, _i32, _V, _V, _i64, _dbl],
    "rpp_gb_log_to_lie": [_vp, _vp, _vp, _i32, _V, _P, _i32, _i32, _i64, _dbl],
    "rpp_gb_lie_to_tensor_exp": [_vp, _vp, _vp, _i32, _P, _P, _V, _i32, _i32, _i64, _dbl],
    "rpp_gb_lie_basis": [_i32, _i32, _I64P, _I64P, _I64P],
    "rpp_gb_conversion_matrix": [_i32, _i32, _i32, _I64P, _I64P, _I64P, _I64P, _I64P, _DBLP],
    "rpp_gb_signature": [_vp, _vp, _i32, _vp, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp],
    "rpp_gb_signature_backward": [_vp, _vp, _i32, _vp, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp],
    "rpp_gb_signature_static_scratch": [_vp, _vp, _i32, _vp, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp],
    "rpp_gb_signature_host": [_vp, _vp, _i32, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64],
    "rpp_gb_fma_peak": [_i32, _i32, _DBLP],
    "rpp_gb_signature_tune": [_vp, _vp, _i32, _vp, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp,
                              ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float)],
    "rpp_gb_signature_with_schedule": [_vp, _vp, _i32, _vp, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i32],
    "rpp_gb_signature_group": [_vp, ctypes.POINTER(SignatureJobArg), _i32, _i32],
    "rpp_gb_exp_letter_vjp": [_vp, _vp, _i32, _vp, _i64, _vp, _i64, _vp, _i64, _i64],
}
RESTYPES = {"rpp_gb_last_error_string": ctypes.c_char_p, "rpp_gb_version": ctypes.c_char_p}


def build(jobs: int = 8) -> None:
    """Compile the CUDA library for sm_103a (nvcc; no GPU needed)."""
    subprocess.run(["make", "-s", "-j", str(jobs), "-C", PKG_DIR], check=True)


def load(path: str = LIB_PATH):
    """Load the shared library once; raise if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(
                    f"{path} is missing: build the CUDA extension first "
                    "(make -C rough-path-primitives_gb300); there is no CPU fallback")
            lib = ctypes.CDLL(path)
            for name, argtypes in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = argtypes
                fn.restype = RESTYPES.get(name, ctypes.c_int)
            _lib = lib
        return _lib
