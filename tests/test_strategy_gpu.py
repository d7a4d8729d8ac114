"""The C++ drop-in on the GPU: tests/cpp/strategy_gpu_parity.cpp calls the
reference's own operation front ends (rpp::ops::<op>) with GB300Strategy on
device buffers -- linked to the real librpp_gb300.so -- and with the
reference's CPU SingleThreadStrategy on host copies of the same inputs, and
prints the largest relative difference per call.  This is the path a
reference user takes after changing only the strategy type.  Needs the
reference's headers (baseline/_ref, or the directory named by RPP_REFERENCE)."""
import importlib
import os
import subprocess

import pytest

from _helpers import TOL_F64

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_INCLUDE = os.path.join(os.environ.get("RPP_REFERENCE", os.path.join(ROOT, "baseline", "_ref")), "include")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
LIB_DIR = os.path.join(ROOT, "rough-path-primitives_gb300", "_build")

# integer-exact operations: a signed reversal of coefficients
EXACT = {"tensor_antipode", "tensor_reflect"}


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    if not os.path.isdir(os.path.join(REF_INCLUDE, "rpp")):
        pytest.skip("reference headers not installed")
    importlib.import_module("rough-path-primitives_gb300").library()  # builds nothing; fails loudly if missing
    exe = tmp_path_factory.mktemp("strategy_gpu") / "parity"
    cmd = ["g++", "-std=c++17", "-O2", "-I", REF_INCLUDE, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "rough-path-primitives_gb300", "include"), "-I", os.path.join(CUDA_HOME, "include"),
           os.path.join(ROOT, "tests", "cpp", "strategy_gpu_parity.cpp"), "-o", str(exe),
           "-L" + LIB_DIR, "-Wl,-rpath," + LIB_DIR, "-lrpp_gb300",
           "-L" + os.path.join(CUDA_HOME, "lib64"), "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64"), "-lcudart"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    out = {}
    for line in res.stdout.splitlines():
        name, _, value = line.partition(" ")
        out[name] = value
    return out


def test_every_call_ran(results):
    assert "failures=0" in results, results
    expected = {"ft_mul", "ft_fma", "ft_inplace_fma_abc", "ft_inplace_fma_bca", "ft_inplace_mul", "ft_exp",
                "ft_fmexp", "ft_log", "ft_adj_lmul", "ft_adj_rmul", "tensor_antipode", "tensor_reflect", "st_mul",
                "st_adj_mul", "left_hs_mul", "tensor_pairing", "tensor_to_lie", "lie_to_tensor", "signature"}
    assert expected <= set(results), sorted(expected - set(results))


@pytest.mark.parametrize("op", ["ft_mul", "ft_fma", "ft_inplace_fma_abc", "ft_inplace_fma_bca", "ft_inplace_mul",
                                "ft_exp", "ft_fmexp", "ft_log", "ft_adj_lmul", "ft_adj_rmul", "tensor_antipode",
                                "tensor_reflect", "st_mul", "st_adj_mul", "left_hs_mul", "tensor_pairing",
                                "tensor_to_lie", "lie_to_tensor", "signature"])
def test_gb300_strategy_matches_reference_cpu_strategy(results, op):
    diff = float(results[op])
    assert diff <= (0.0 if op in EXACT else TOL_F64), f"{op}: relative difference {diff:.3e}"
