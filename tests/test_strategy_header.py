"""The C++ drop-in (rpp/gpu/gb300/strategy.hpp) compiles against the
reference's headers and turns the reference's own operation front ends into
the right C-ABI calls.  Built with g++ against a recording test double of the
C ABI, so no GPU is needed; skipped where the reference's headers are absent
(they are installed into baseline/_ref, or named by RPP_REFERENCE)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_INCLUDE = os.path.join(os.environ.get("RPP_REFERENCE", os.path.join(ROOT, "baseline", "_ref")), "include")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def calls(tmp_path_factory):
    if not os.path.isdir(os.path.join(REF_INCLUDE, "rpp")):
        pytest.skip("reference headers not available")
    out = tmp_path_factory.mktemp("strategy") / "driver"
    cmd = ["g++", "-std=c++17", "-O0", "-I", REF_INCLUDE, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "rough-path-primitives_gb300", "include"), "-I", os.path.join(CUDA_HOME, "include"),
           os.path.join(ROOT, "tests", "cpp", "strategy_driver.cpp"), os.path.join(ROOT, "tests", "cpp", "mock_capi.cpp"),
           "-o", str(out), "-L" + os.path.join(CUDA_HOME, "lib64"), "-lcudart"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    res = subprocess.run([str(out)], capture_output=True, text=True,
                         env={**os.environ, "LD_LIBRARY_PATH": os.path.join(CUDA_HOME, "lib64")})
    assert res.returncode == 0, res.stdout + res.stderr
    return res.stdout.splitlines()


def test_plan_created_once_per_basis(calls):
    assert [c for c in calls if c.startswith("plan_create")] == ["plan_create W=3 D=4 dev=2"]


def test_products(calls):
    assert "ft_mul dtype=1 n=4 out{s=128,0..4} lhs{s=128,1..2} rhs{s=121,1..1} a=0 b=0.5" in calls
    assert "ft_fma dtype=1 n=4 out{s=128,0..4} a{s=128,1..2} b{s=128,0..4} c{s=121,1..1} a=0.25 b=2" in calls
    assert "ft_inplace_fma dtype=1 n=4 kind=1 a{s=128,0..4} b{s=121,1..1} c{s=128,1..2} a=1 b=0.5" in calls
    assert "ft_inplace_mul dtype=1 n=4 lhs{s=128,0..4} rhs{s=121,1..1} a=0 b=3" in calls


def test_intermediates_and_adjoints(calls):
    assert "ft_exp dtype=1 n=4 out{s=128,0..4} arg{s=128,1..2} a=0 b=0" in calls
    assert "ft_fmexp dtype=1 n=4 out{s=128,0..4} x{s=128,1..2} y{s=121,1..1} a=0 b=0" in calls
    assert "ft_log dtype=1 n=4 out{s=128,0..4} arg{s=128,1..2} a=0 b=0" in calls
    assert "ft_adj_lmul dtype=1 n=4 out{s=128,1..2} x{s=128,0..4} y{s=121,1..1} a=0 b=0" in calls
    assert "ft_adj_rmul dtype=1 n=4 out{s=128,1..2} x{s=128,0..4} y{s=121,1..1} a=0 b=0" in calls
    assert "tensor_antipode dtype=1 n=4 policy=1 out{s=128,0..4} arg{s=128,1..2} a=0 b=0" in calls
    assert "tensor_antipode dtype=1 n=4 policy=0 out{s=128,0..4} arg{s=128,1..2} a=0 b=0" in calls


def test_tensor_to_lie_uses_begin_relative_views_and_caches_matrix(calls):
    uploads = [c for c in calls if c.startswith("matrix_create")]
    # the t2l matrix once (the fused log-to-Lie call reuses it), then the l2t matrix once
    assert uploads == ["matrix_create fmt=1 outer=121 inner=32 nnz=109 dev=2",
                       "matrix_create fmt=1 outer=32 inner=121 nnz=133 dev=2"]
    spmv = [c for c in calls if c.startswith("spmv")]
    assert len(spmv) == 2
    assert spmv[0] == "spmv dtype=1 n=4 out{s=40,begin=1,size=32} arg{s=128,begin=0,size=121} a=1 b=0"


def test_signature_entry(calls):
    assert "signature dtype=1 n=4 len=16 offsets=0 sig_stride=121 seed=0 grad=0" in calls
    assert calls[-1] == "failures=0"


def test_shuffle_algebra(calls):
    assert "st_mul dtype=1 n=4 out{s=128,0..4} x{s=128,1..2} y{s=121,1..1} a=0 b=0.5" in calls
    assert "st_fma dtype=1 n=4 out{s=128,0..4} a{s=128,1..2} b{s=128,0..4} c{s=121,1..1} a=0.25 b=2" in calls
    assert "st_inplace_fma dtype=1 n=4 a{s=128,0..4} b{s=121,1..1} c{s=128,1..2} a=1 b=0.5" in calls
    assert "st_adj_mul dtype=1 n=4 out{s=128,1..2} x{s=128,0..4} y{s=121,1..1} a=0 b=0" in calls
    assert "left_hs_mul dtype=1 n=4 out{s=128,0..4} x{s=128,1..2} y{s=121,1..1} a=0 b=3" in calls
    assert "left_hs_adj_lmul dtype=1 n=4 out{s=128,1..2} x{s=128,0..4} y{s=121,1..1} a=0 b=1" in calls
    assert "left_hs_adj_rmul dtype=1 n=4 out{s=128,1..2} x{s=128,0..4} y{s=121,1..1} a=0 b=2" in calls
    assert "tensor_pairing dtype=1 n=4 result=set f{s=128,1..2} arg{s=121,1..1} a=0 b=0" in calls



def test_fused_lie_steps(calls):
    """The C++ helpers for the fused steps pass the views' ranges and the
    cached matrices (the l2t matrix is uploaded once, like the t2l one)."""
    assert "log_to_lie dtype=1 n=4 out{b=1,n=32} degrees=0..4 arg{s=128,0..4} a=0.5 b=0" in calls
    assert "lie_to_tensor_exp dtype=1 n=4 out{s=128,0..4} arg{b=1,n=32} degrees=0..4 a=1 b=0" in calls
    assert ("lie_to_tensor_exp dtype=1 n=4 out{s=128,0..4} mult{s=128,0..4} arg{b=1,n=32} degrees=0..4 a=2 b=0"
            in calls)
    assert sum(c.startswith("matrix_create") for c in calls) == 2
