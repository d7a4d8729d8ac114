"""Parity of the per-operation sm_103a kernels with the oracle and with the
reference's golden outputs, through the C ABI (ctypes).

FP64 must agree to 1e-12 relative (floor 1) and FP32 to 1e-5, both measured
against FP64 expectations (tests/rpp/cpu/single_thread/ops/
cpu_typed_ft_ops_test_helper.hpp:33-36, :261-273).  Antipode/reflect are pure
index permutations and must be bit-exact."""
import importlib
import os

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F32, TOL_F64, assert_close

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")

DTYPES = [(torch.float64, TOL_F64), (torch.float32, TOL_F32)]


@pytest.fixture(scope="module")
def ops_golden(golden_dir):
    return np.load(os.path.join(golden_dir, "ops_w3d4.npz"))


def _cases(z, op):
    keys = sorted({k.split("/")[1] for k in z.files if k.startswith(op + "/")}, key=int)
    return [{k.split("/")[2]: z[k] for k in z.files if k.startswith(f"{op}/{i}/")} for i in keys]


def dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def tb(t, dim, rng):
    return pkg.make_tensor_batch(t, dim, int(rng[0]), int(rng[1]))


@pytest.mark.parametrize("dtype,tol", DTYPES)
def test_ft_mul_golden(ops_golden, dtype, tol):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    for c in _cases(ops_golden, "ft_mul"):
        r = c["ranges"]
        out = dev(c["init"], dtype)
        n = out.shape[0]
        assert pkg.ft_mul(st, None, tb(out, dim, r[0]), tb(dev(c["lhs"], dtype), dim, r[1]),
                          tb(dev(c["rhs"], dtype), dim, r[2]), basis, n, float(c["beta"]))
        assert_close(host(out), c["out"], tol, f"ft_mul {r.tolist()}")


@pytest.mark.parametrize("dtype,tol", DTYPES)
def test_ft_fma_golden(ops_golden, dtype, tol):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    for c in _cases(ops_golden, "ft_fma"):
        r = c["ranges"]
        out = dev(c["init"], dtype)
        n = out.shape[0]
        assert pkg.ft_fma(st, None, tb(out, dim, r[0]), tb(dev(c["a"], dtype), dim, r[1]),
                          tb(dev(c["b"], dtype), dim, r[2]), tb(dev(c["c"], dtype), dim, r[3]), basis, n,
                          float(c["alpha"]), float(c["beta"]))
        assert_close(host(out), c["out"], tol, f"ft_fma {r.tolist()}")


@pytest.mark.parametrize("dtype,tol", DTYPES)
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_ft_inplace_fma_golden(ops_golden, dtype, tol, kind):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    for c in _cases(ops_golden, f"ft_inplace_fma{kind}"):
        r = c["ranges"]
        a = dev(c["a"], dtype)
        n = a.shape[0]
        assert pkg.ft_inplace_fma(kind, st, None, tb(a, dim, r[0]), tb(dev(c["b"], dtype), dim, r[1]),
                                  tb(dev(c["c"], dtype), dim, r[2]), basis, n, float(c["alpha"]), float(c["beta"]))
        assert_close(host(a), c["out"], tol, f"inplace_fma{kind} {r.tolist()}")


@pytest.mark.parametrize("dtype,tol", DTYPES)
def test_ft_inplace_mul_golden(ops_golden, dtype, tol):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    for c in _cases(ops_golden, "ft_inplace_mul"):
        r = c["ranges"]
        a = dev(c["a"], dtype)
        assert pkg.ft_inplace_mul(st, None, tb(a, dim, r[0]), tb(dev(c["b"], dtype), dim, r[1]), basis,
                                  a.shape[0], float(c["beta"]))
        assert_close(host(a), c["out"], tol, f"inplace_mul {r.tolist()}")


@pytest.mark.parametrize("dtype,tol", DTYPES)
@pytest.mark.parametrize("op", ["ft_exp", "ft_log"])
def test_exp_log_golden(ops_golden, dtype, tol, op):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    for c in _cases(ops_golden, op):
        r = c["ranges"]
        out = dev(c["init"], dtype)
        assert getattr(pkg, op)(st, None, tb(out, dim, r[0]), tb(dev(c["arg"], dtype), dim, r[1]), basis,
                                out.shape[0])
        assert_close(host(out), c["out"], tol, f"{op} {r.tolist()}")


@pytest.mark.parametrize("dtype,tol", DTYPES)
def test_ft_fmexp_golden(ops_golden, dtype, tol):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    for c in _cases(ops_golden, "ft_fmexp"):
        r = c["ranges"]
        out = dev(c["init"], dtype)
        assert pkg.ft_fmexp(st, None, tb(out, dim, r[0]), tb(dev(c["mult"], dtype), dim, r[1]),
                            tb(dev(c["x"], dtype), dim, r[2]), basis, out.shape[0])
        assert_close(host(out), c["out"], tol, f"fmexp {r.tolist()}")


@pytest.mark.parametrize("dtype,tol", DTYPES)
@pytest.mark.parametrize("left", [1, 0])
def test_adjoints_golden(ops_golden, dtype, tol, left):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    fn = pkg.ft_adj_lmul if left else pkg.ft_adj_rmul
    for c in _cases(ops_golden, "ft_adj_lmul" if left else "ft_adj_rmul"):
        r = c["ranges"]
        out = dev(c["init"], dtype)
        assert fn(st, None, tb(out, dim, r[0]), tb(dev(c["op"], dtype), dim, r[1]), tb(dev(c["arg"], dtype), dim, r[2]),
                  basis, out.shape[0])
        assert_close(host(out), c["out"], tol, f"adjoint left={left} {r.tolist()}")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("signed", [1, 0])
def test_antipode_bit_exact(ops_golden, dtype, signed):
    W, D = int(ops_golden["width"]), int(ops_golden["depth"])
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    fn = pkg.tensor_antipode if signed else pkg.tensor_reflect
    for c in _cases(ops_golden, "tensor_antipode" if signed else "tensor_reflect"):
        r = c["ranges"]
        out = dev(c["init"], dtype)
        assert fn(st, None, tb(out, dim, r[0]), tb(dev(c["arg"], dtype), dim, r[1]), basis, out.shape[0])
        expect = c["out"].astype(np.float32).astype(np.float64) if dtype == torch.float32 else c["out"]
        assert np.array_equal(host(out), expect)


# Larger random cases against the oracle, including the benchmark shapes.
RANDOM_SHAPES = [(4, 4, 64), (5, 5, 8), (2, 8, 8), (8, 3, 8), (16, 3, 2), (1, 5, 4), (3, 0, 4), (6, 4, 3),
                 (2, 12, 3)]  # (W2 D12: the adjoints stage the op only)


@pytest.mark.parametrize("W,D,n", RANDOM_SHAPES)
def test_products_random(orc, W, D, n):
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    rng = np.random.default_rng(W * 100 + D)
    full = (0, D)
    st = pkg.GB300Strategy(torch.float64)
    x, y, z = (rng.uniform(-1, 1, (n, dim)) for _ in range(3))
    for rr in [(full, full, full), ((1, D), (0, max(0, D - 2)), (1, D)), ((min(2, D), D), (1, 1), (0, D))]:
        out = torch.zeros(n, dim, dtype=torch.float64, device="cuda")
        assert pkg.ft_mul(st, None, tb(out, dim, rr[0]), tb(dev(x, torch.float64), dim, rr[1]),
                          tb(dev(y, torch.float64), dim, rr[2]), basis, n, 0.5)
        e = np.zeros((n, dim))
        orc.ft_mul(W, D, e, x, y, rr, 0.5)
        assert_close(host(out), e, TOL_F64, f"ft_mul W{W}D{D} {rr}")
        for kind in range(3):
            a = dev(z, torch.float64)
            assert pkg.ft_inplace_fma(kind, st, None, tb(a, dim, rr[0]), tb(dev(x, torch.float64), dim, rr[1]),
                                      tb(dev(y, torch.float64), dim, rr[2]), basis, n, 0.25, 0.75)
            e = z.copy()
            orc.ft_inplace_fma(W, D, kind, e, x, y, rr, 0.25, 0.75)
            assert_close(host(a), e, TOL_F64, f"inplace kind {kind} W{W}D{D} {rr}")


@pytest.mark.parametrize("W,D,n", RANDOM_SHAPES)
def test_intermediates_random(orc, W, D, n):
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    rng = np.random.default_rng(7 + W + D)
    st = pkg.GB300Strategy(torch.float64)
    scale = 0.5 / max(1, W)
    x = rng.uniform(-1, 1, (n, dim)) * scale
    m = rng.uniform(-1, 1, (n, dim))
    full = (0, D)
    out = torch.zeros(n, dim, dtype=torch.float64, device="cuda")
    assert pkg.ft_exp(st, None, tb(out, dim, full), tb(dev(x, torch.float64), dim, full), basis, n)
    e = np.zeros((n, dim))
    orc.ft_exp(W, D, e, x, (full, full))
    assert_close(host(out), e, TOL_F64, "exp")
    assert pkg.ft_fmexp(st, None, tb(out, dim, full), tb(dev(m, torch.float64), dim, full),
                        tb(dev(x, torch.float64), dim, full), basis, n)
    orc.ft_fmexp(W, D, e, m, x, (full, full, full))
    assert_close(host(out), e, TOL_F64, "fmexp")
    xl = x.copy()
    xl[:, 0] = 1.0
    assert pkg.ft_log(st, None, tb(out, dim, full), tb(dev(xl, torch.float64), dim, full), basis, n)
    orc.ft_log(W, D, e, xl, (full, full))
    assert_close(host(out), e, TOL_F64, "log")
    for left in (1, 0):
        fn = pkg.ft_adj_lmul if left else pkg.ft_adj_rmul
        assert fn(st, None, tb(out, dim, full), tb(dev(m, torch.float64), dim, full),
                  tb(dev(x, torch.float64), dim, full), basis, n)
        orc.ft_adj_mul(W, D, left, e, m, x, (full, full, full))
        assert_close(host(out), e, TOL_F64, f"adjoint left={left}")


def test_exp_log_roundtrip_and_adjoint_pairing():
    """log(exp(x)) = x; <adj_lmul(op, arg), y> = <arg, op (x) y>
    (tests/rpp/cpu/single_thread/ops/ft_exp_log_tests.cpp, ft_adj_lmul_tests.cpp:416)."""
    W, D, n = 4, 5, 16
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    full = (0, D)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (n, dim)) * 0.2
    x[:, 0] = 0
    ex = torch.zeros(n, dim, dtype=torch.float64, device="cuda")
    lg = torch.zeros_like(ex)
    assert pkg.ft_exp(st, None, tb(ex, dim, full), tb(dev(x, torch.float64), dim, full), basis, n)
    assert pkg.ft_log(st, None, tb(lg, dim, full), tb(ex, dim, full), basis, n)
    assert_close(host(lg), x, TOL_F64, "log(exp(x))")
    op, arg, y = (dev(rng.uniform(-1, 1, (n, dim)), torch.float64) for _ in range(3))
    adj = torch.zeros_like(op)
    prod = torch.zeros_like(op)
    assert pkg.ft_adj_lmul(st, None, tb(adj, dim, full), tb(op, dim, full), tb(arg, dim, full), basis, n)
    assert pkg.ft_mul(st, None, tb(prod, dim, full), tb(op, dim, full), tb(y, dim, full), basis, n)
    lhs = (adj * y).sum(1)
    rhs = (arg * prod).sum(1)
    assert_close(host(lhs), host(rhs), 1e-12, "adjoint pairing")


@pytest.mark.parametrize("dtype,tol", DTYPES)
def test_helpers(dtype, tol):
    W, D, n = 3, 3, 5
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(dtype)
    src = torch.arange(n * dim, dtype=dtype, device="cuda").reshape(n, dim)
    out = torch.full((n, dim), 7.0, dtype=dtype, device="cuda")
    assert pkg.vector_assign(st, None, tb(out, dim, (1, 2)), tb(src, dim, (2, 3)), basis, n)
    o = host(out)
    assert (o[:, 0] == 7).all() and (o[:, 1:4] == 0).all()
    assert np.array_equal(o[:, 4:13], host(src)[:, 4:13]) and (o[:, 13:] == 7).all()
    assert pkg.tensor_set_identity(st, None, tb(out, dim, (0, 1)), basis, n, 2.0)
    o = host(out)
    assert (o[:, 0] == 2).all() and (o[:, 1:4] == 0).all()
    assert pkg.tensor_add_identity(st, None, tb(out, dim, (0, 3)), basis, n, 0.5)
    assert (host(out)[:, 0] == 2.5).all()
    assert pkg.vector_set_constant(st, None, tb(out, dim, (2, 3)), basis, n, -1.0)
    assert (host(out)[:, 4:] == -1).all()


@pytest.mark.parametrize("dtype,tol", DTYPES)
@pytest.mark.parametrize("wd", [(3, 4), (5, 5)])
def test_lie_conversions_golden(golden_dir, dtype, tol, wd):
    """tensor_to_lie / lie_to_tensor with NaN-poisoned outputs and sentinel
    guards (tests/rpp/lie_tensor_conversion_test_helper.hpp:19-81)."""
    z = np.load(os.path.join(golden_dir, f"lie_{wd[0]}_{wd[1]}.npz"))
    W, D = wd
    tbasis, lbasis = pkg.TensorBasis(W, D), pkg.LieBasis(W, D)
    st = pkg.GB300Strategy(dtype)
    t2l, l2t = pkg.make_t2l_matrix(lbasis), pkg.make_l2t_matrix(lbasis)
    n, ts, dim = z["t2l_arg"].shape[0], lbasis.true_size(), tbasis.size()
    # output with one guard slot on each side of every batch element
    buf = torch.full((n, ts + 2), float("nan"), dtype=dtype, device="cuda")
    buf[:, 0] = 7.0
    buf[:, -1] = 7.0
    out = pkg.make_lie_batch(buf[:, 1:], ts + 2, 1, D)
    assert pkg.tensor_to_lie(st, None, out, pkg.make_tensor_batch(dev(z["t2l_arg"], dtype), dim, 0, D), lbasis,
                             tbasis, n, t2l)
    got = host(buf)
    assert (got[:, 0] == 7).all() and (got[:, -1] == 7).all() and np.isnan(got[:, 1]).all()
    assert_close(got[:, 2:-1], z["t2l_out"][:, 1:], tol, "tensor_to_lie")
    tbuf = torch.full((n, dim + 2), float("nan"), dtype=dtype, device="cuda")
    tbuf[:, 0] = 7.0
    tbuf[:, -1] = 7.0
    assert pkg.lie_to_tensor(st, None, pkg.make_tensor_batch(tbuf[:, 1:], dim + 2, 0, D),
                             pkg.make_lie_batch(dev(z["l2t_arg"], dtype), ts, 1, D), tbasis, lbasis, n, l2t)
    got = host(tbuf)
    assert (got[:, 0] == 7).all() and (got[:, -1] == 7).all()
    assert_close(got[:, 1:-1], z["l2t_out"], tol, "lie_to_tensor")


def test_invalid_arguments_are_reported():
    basis = pkg.TensorBasis(3, 3)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    t = torch.zeros(4, dim, dtype=torch.float64, device="cuda")
    err = pkg.ft_mul(st, None, pkg.make_tensor_batch(t, dim, -1, 3), pkg.make_tensor_batch(t, dim, 0, 3),
                     pkg.make_tensor_batch(t, dim, 0, 3), basis, 4)
    assert not err and err.code == pkg.ErrorCode.InvalidArgument and "min_degree" in err.message
    err = pkg.ft_fmexp(st, None, pkg.make_tensor_batch(t, dim, 0, 3), pkg.make_tensor_batch(t, dim, 0, 3),
                       pkg.make_tensor_batch(t, dim, 1, 1), basis, 4)
    assert not err and err.code == pkg.ErrorCode.InvalidArgument
    assert pkg.ft_mul(st, None, pkg.make_tensor_batch(t, dim, 0, 3), pkg.make_tensor_batch(t, dim, 0, 3),
                      pkg.make_tensor_batch(t, dim, 0, 3), basis, 0)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, TOL_F64), (torch.float32, TOL_F32)])
@pytest.mark.parametrize("W,D,n", [(4, 4, 1024), (3, 5, 700), (5, 3, 1500)])
def test_products_large_batches(orc, dtype, tol, W, D, n):
    """Batches of several tensors per SM (a full wave and more of the product
    kernel): ft_mul with beta = 1 and beta != 1 and degree ranges, and ft_fma
    with an addend, against the oracle; odd batch strides put every other row
    off the 16-byte alignment of the bulk copies."""
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    stride = dim + 3
    rng = np.random.default_rng(W * 10 + D + n)
    st = pkg.GB300Strategy(dtype)
    x, y, z = (rng.uniform(-1, 1, (n, stride)) for _ in range(3))
    full = (0, D)
    for rr, beta in [((full, full, full), 1.0), (((1, D), (0, max(0, D - 2)), (1, D)), 0.5)]:
        out = torch.zeros(n, stride, dtype=dtype, device="cuda")
        err = pkg.ft_mul(st, None, tb(out, stride, rr[0]), tb(dev(x, dtype), stride, rr[1]),
                         tb(dev(y, dtype), stride, rr[2]), basis, n, beta)
        assert err, err.message
        e = np.zeros((n, stride))
        orc.ft_mul(W, D, e, x, y, rr, beta)
        assert_close(host(out)[:, :dim], e[:, :dim], tol, f"ft_mul W{W}D{D} n{n} {rr}")
    out = torch.zeros(n, stride, dtype=dtype, device="cuda")
    err = pkg.ft_fma(st, None, tb(out, stride, full), tb(dev(z, dtype), stride, full), tb(dev(x, dtype), stride, full),
                     tb(dev(y, dtype), stride, full), basis, n, 0.25, 0.75)
    assert err, err.message
    e = np.zeros((n, stride))
    orc.ft_fma(W, D, e, z, x, y, (full, full, full, full), 0.25, 0.75)
    assert_close(host(out)[:, :dim], e[:, :dim], tol, f"ft_fma W{W}D{D} n{n}")


def test_dependent_products_in_a_graph(orc):
    """A chain in which every product reads the one before it -- with an
    in-place product and a non-product kernel in between -- gives the oracle's
    chain, eagerly and from a CUDA graph, and the two agree bit for bit."""
    W, D, n = 4, 4, 1024
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    full = (0, D)
    rng = np.random.default_rng(404)
    a_h, b_h = (rng.uniform(-0.5, 0.5, (n, dim)) for _ in range(2))
    st = pkg.GB300Strategy(torch.float64)
    a, b = dev(a_h, torch.float64), dev(b_h, torch.float64)
    x1, x2, x4 = (torch.zeros(n, dim, dtype=torch.float64, device="cuda") for _ in range(3))

    def chain(cfg):
        t = lambda v: tb(v, dim, full)  # noqa: E731
        pkg.ft_mul(st, cfg, t(x1), t(a), t(b), basis, n).raise_if_failed()
        pkg.ft_mul(st, cfg, t(x2), t(x1), t(b), basis, n).raise_if_failed()
        pkg.ft_inplace_mul(st, cfg, t(x2), t(a), basis, n).raise_if_failed()
        x2.mul_(0.5)
        pkg.ft_fma(st, cfg, t(x4), t(x2), t(x1), t(x2), basis, n).raise_if_failed()

    chain(None)
    eager = host(x4).copy()
    # the oracle's chain
    e1, e2, e4 = (np.zeros((n, dim)) for _ in range(3))
    rr = (full, full, full)
    orc.ft_mul(W, D, e1, a_h, b_h, rr)
    orc.ft_mul(W, D, e2, e1, b_h, rr)
    e3 = np.zeros((n, dim))
    orc.ft_mul(W, D, e3, e2, a_h, rr)
    e3 *= 0.5
    orc.ft_fma(W, D, e4, e3, e1, e3, (full, full, full, full))
    assert_close(eager, e4, TOL_F64, "dependent chain, eager")
    # the same chain captured in a graph and replayed
    for v in (x1, x2, x4):
        v.zero_()
    cap = torch.cuda.Stream()
    cap.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(cap):
        cfg = pkg.DeviceLaunchConfig(cap)
        with torch.cuda.graph(graph, stream=cap):
            chain(cfg)
    torch.cuda.current_stream().wait_stream(cap)
    for v in (x1, x2, x4):
        v.fill_(float("nan"))
    graph.replay()
    assert np.array_equal(host(x4), eager)
