"""Shuffle-algebra operations and tensor_pairing on the GPU against the oracle
and the reference's golden outputs, through the Python mirror of the
reference's operation API (which calls the C ABI).

Reference behaviour checked (include/rpp/cpu/single_thread/operations/basic/
st_*.hpp, left_hs_*.hpp, tensor_pairing.hpp and the reference's tests under
tests/rpp/cpu/single_thread/ops/): degrees outside an input view are never
read (they hold NaN here), coefficients outside the output view are never
written (they keep their initial bits), and FP64 results agree to 1e-12
relative (floor one), FP32 to 1e-5."""
import importlib
import os

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F32, TOL_F64, assert_close, shuffle_cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


def _r(ranges):
    return tuple(tuple(int(v) for v in r) for r in ranges)


def _nan_outside(a, W, D, rng):
    """Copy of a with NaN in every degree outside rng (forbidden reads)."""
    a = a.copy()
    db = O.degree_begin(W, D)
    for n in range(D + 1):
        if not (rng[0] <= n <= rng[1]):
            a[:, db[n]:db[n + 1]] = np.nan
    return a


def run_op(name, W, D, out_init, inputs, ranges, dtype=torch.float64, **scal):
    """Run one op on the GPU.  inputs: numpy arrays in the C-ABI argument
    order after `out`; ranges: (out, *inputs) degree ranges."""
    basis = pkg.TensorBasis(W, D)
    st = pkg.GB300Strategy(dtype)
    n, dim = out_init.shape
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)  # noqa: E731
    out = dev(out_init)
    ins = [dev(_nan_outside(a, W, D, r)) for a, r in zip(inputs, ranges[1:])]
    mk = lambda t, r: pkg.make_tensor_batch(t, dim, r[0], r[1])  # noqa: E731
    ob = mk(out, ranges[0])
    ib = [mk(t, r) for t, r in zip(ins, ranges[1:])]
    fn = getattr(pkg, name)
    if name == "st_inplace_fma":
        err = fn(st, None, ob, ib[0], ib[1], basis, n, **scal)
    else:
        err = fn(st, None, ob, *ib, basis, n, **scal)
    assert err, f"{name}: {err}"
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


def _check_untouched(got, init, out_range, W, D):
    db = O.degree_begin(W, D)
    lo, hi = out_range
    outside = np.ones(got.shape[1], bool)
    if lo <= min(hi, D):
        outside[db[lo]:db[min(hi, D) + 1]] = False
    assert np.array_equal(got[:, outside].view(np.int64), init[:, outside].view(np.int64)), "wrote outside out's range"


@pytest.fixture(scope="module")
def sh(golden_dir):
    return np.load(os.path.join(golden_dir, "shuffle_w3d4.npz"))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_golden_products(sh, dtype):
    tol = TOL_F64 if dtype == torch.float64 else TOL_F32
    x, y, z, init = sh["inputs/x"], sh["inputs/y"], sh["inputs/z"], sh["inputs/init"]
    for c in shuffle_cases(sh, "st_mul"):
        rr = _r(c["ranges"])
        got = run_op("st_mul", 3, 4, init, [x, y], rr, dtype, beta=float(c["beta"]))
        assert_close(got, c["out"], tol, f"st_mul {rr}")
        _check_untouched(got, init, rr[0], 3, 4)
    for c in shuffle_cases(sh, "st_fma"):
        rr = _r(c["ranges"])
        got = run_op("st_fma", 3, 4, init, [z, x, y], rr, dtype, alpha=float(c["alpha"]), beta=float(c["beta"]))
        assert_close(got, c["out"], tol, f"st_fma {rr}")
        _check_untouched(got, init, rr[0], 3, 4)
    for c in shuffle_cases(sh, "st_inplace_fma"):
        rr = _r(c["ranges"])
        got = run_op("st_inplace_fma", 3, 4, z, [x, y], rr, dtype, alpha=float(c["alpha"]), beta=float(c["beta"]))
        assert_close(got, c["out"], tol, f"st_inplace_fma {rr}")
        _check_untouched(got, z, rr[0], 3, 4)
    for c in shuffle_cases(sh, "left_hs_mul"):
        rr = _r(c["ranges"])
        got = run_op("left_hs_mul", 3, 4, init, [x, y], rr, dtype, beta=float(c["beta"]))
        assert_close(got, c["out"], tol, f"left_hs_mul {rr}")
        _check_untouched(got, init, rr[0], 3, 4)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_golden_adjoints(sh, dtype):
    tol = TOL_F64 if dtype == torch.float64 else TOL_F32
    x, y, init = sh["inputs/x"], sh["inputs/y"], sh["inputs/init"]
    for c in shuffle_cases(sh, "st_adj_mul"):
        rr = _r(c["ranges"])
        got = run_op("st_adj_mul", 3, 4, init, [x, y], rr, dtype)
        assert_close(got, c["out"], tol, f"st_adj_mul {rr}")
        _check_untouched(got, init, rr[0], 3, 4)
    for c in shuffle_cases(sh, "left_hs_adj_lmul"):
        o, f, a = _r(c["ranges"])  # (out, fixed integrator x, cotangent y)
        got = run_op("left_hs_adj_lmul", 3, 4, init, [x, y], (o, f, a), dtype)
        assert_close(got, c["out"], tol, f"left_hs_adj_lmul {(o, f, a)}")
        _check_untouched(got, init, o, 3, 4)
    for c in shuffle_cases(sh, "left_hs_adj_rmul"):
        o, f, a = _r(c["ranges"])  # (out, fixed integrand x, cotangent y)
        got = run_op("left_hs_adj_rmul", 3, 4, init, [y, x], (o, a, f), dtype)
        assert_close(got, c["out"], tol, f"left_hs_adj_rmul {(o, f, a)}")
        _check_untouched(got, init, o, 3, 4)


@pytest.mark.parametrize("W,D", [(1, 4), (2, 2), (4, 0)])
def test_golden_small_bases(sh, W, D):
    key = f"small_{W}_{D}"
    a, b, init = sh[f"{key}/a"], sh[f"{key}/b"], sh[f"{key}/init"]
    full = ((0, D),) * 3
    for name in ("st_mul", "left_hs_mul", "st_adj_mul", "left_hs_adj_lmul", "left_hs_adj_rmul"):
        got = run_op(name, W, D, init, [a, b], full)
        assert_close(got, sh[f"{key}/{name}"], TOL_F64, f"{name} W{W} D{D}")


def test_golden_pairing(sh):
    x, y = sh["inputs/x"], sh["inputs/y"]
    basis = pkg.TensorBasis(3, 4)
    st = pkg.GB300Strategy(torch.float64)
    for c in shuffle_cases(sh, "tensor_pairing"):
        fr, ar = _r(c["ranges"])
        f = torch.from_numpy(_nan_outside(x, 3, 4, fr)).cuda()
        a = torch.from_numpy(_nan_outside(y, 3, 4, ar)).cuda()
        res = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        assert pkg.tensor_pairing(st, None, pkg.make_scalar_batch(res), pkg.make_tensor_batch(f, 121, *fr),
                                  pkg.make_tensor_batch(a, 121, *ar), basis, 2)
        assert_close(res.cpu().numpy(), c["out"], TOL_F64, f"tensor_pairing {fr} {ar}")


# Larger bases against the oracle: W5 D5 (the staged shared-memory path),
# W2 D8 (deep words, 2^8 subsets), W16 D2, W6 D6 (operands beyond shared
# memory: the global-memory path) and W3 D9 (the 16-letter kernel variant).
SHAPES = [(5, 5, 6), (2, 8, 4), (16, 2, 5), (6, 6, 2), (3, 9, 1)]
RANGE_SETS = {
    "full": lambda D: ((0, D), (0, D), (0, D)),
    "restricted": lambda D: ((1, D - 1), (1, max(1, D - 2)), (0, D - 1)),
}


def _oracle_op(orc, name, W, D, out, x, y, rr, scal):
    if name == "st_mul":
        orc.st_mul(W, D, out, x, y, rr, scal["beta"])
    elif name == "left_hs_mul":
        orc.left_hs_mul(W, D, out, x, y, rr, scal["beta"])
    elif name == "st_inplace_fma":
        orc.st_inplace_fma(W, D, out, x, y, rr, scal["alpha"], scal["beta"])
    elif name == "st_adj_mul":
        orc.st_adj_mul(W, D, out, x, y, rr)
    else:
        orc.left_hs_adjoint(W, D, name.endswith("lmul"), out, x, y, rr, scal["beta"])


OPS = [("st_mul", {"beta": 0.5}), ("left_hs_mul", {"beta": -2.0}), ("st_inplace_fma", {"alpha": 0.5, "beta": 1.5}),
       ("st_adj_mul", {}), ("left_hs_adj_lmul", {"beta": 0.75}), ("left_hs_adj_rmul", {"beta": 0.75})]


@pytest.mark.parametrize("W,D,B", SHAPES)
@pytest.mark.parametrize("which", ["full", "restricted"])
def test_against_oracle(orc, W, D, B, which):
    """A coefficient of these shapes sums up to ~1e5 products (W3 D9) whose
    partial sums grow far beyond the result, so two correct summation orders
    differ by more than 1e-12 of an O(1) coefficient.  Each coefficient is
    therefore checked against |got - want| <= 1e-12 max(1, |want|) + 1e-13 S,
    S = the sum of the absolute values of its terms (the oracle run on |x|,
    |y|, |scalars|).  A missing, extra or wrong term moves a coefficient by a
    whole product, orders of magnitude above this bound."""
    if W == 3 and D == 9 and which == "restricted":
        pytest.skip("one range set is enough for the slowest oracle shape")
    dim = O.tensor_dim(W, D)
    rng = np.random.default_rng(W * 100 + D)
    x, y, z, init = (rng.uniform(-1, 1, (B, dim)) for _ in range(4))
    rr = RANGE_SETS[which](D)
    for name, scal in OPS:
        start = z if name == "st_inplace_fma" else init
        want = start.copy()
        _oracle_op(orc, name, W, D, want, x, y, rr, scal)
        size = start.copy() if name != "st_inplace_fma" else np.abs(z)
        _oracle_op(orc, name, W, D, size, np.abs(x), np.abs(y), rr, {k: abs(v) for k, v in scal.items()})
        got = run_op(name, W, D, start, [x, y], rr, **scal)
        db = O.degree_begin(W, D)
        lo, hi = rr[0][0], min(rr[0][1], D)
        sl = slice(db[lo], db[hi + 1])
        err = np.abs(got[:, sl] - want[:, sl])
        bound = TOL_F64 * np.maximum(1.0, np.abs(want[:, sl])) + 1e-13 * np.abs(size[:, sl])
        worst = float(np.max(err / bound)) if err.size else 0.0
        assert np.all(np.isfinite(got[:, sl])) and worst <= 1.0, f"{name} W{W} D{D} {which}: {worst:.3f} of bound"
        _check_untouched(got, start, rr[0], W, D)


def test_st_fma_without_addend_range(orc):
    """An addend view missing degrees contributes nothing there
    (st_fma.hpp: a.has_degree checks)."""
    W, D, B = 4, 4, 3
    dim = O.tensor_dim(W, D)
    rng = np.random.default_rng(8)
    a, b, c, init = (rng.uniform(-1, 1, (B, dim)) for _ in range(4))
    rr = ((0, D), (2, 3), (0, D), (1, D))
    e = init.copy()
    orc.st_fma(W, D, e, a, b, c, rr, 0.5, 2.0)
    got = run_op("st_fma", W, D, init, [a, b, c], rr, alpha=0.5, beta=2.0)
    assert_close(got, e, TOL_F64, "st_fma")


def _pair(a, b):
    return (a * b).sum(dim=1)


def test_signature_is_a_shuffle_character_full_size():
    """4096 signatures of W5 D5 paths of 256 steps: <S, f sh g> = <S, f><S, g>
    for every f, g whose shuffle product stays within depth 5 (f of degree
    <= 2, g of degree <= 3), through st_mul and tensor_pairing."""
    W, D, B, L = 5, 5, 4096, 256
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    gen = torch.Generator(device="cuda").manual_seed(12)
    incr = torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=gen) / np.sqrt(L)
    sig = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    assert pkg.signature(st, None, incr, basis, B, length=L, out=sig)
    f = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=gen) - 0.5
    g = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=gen) - 0.5
    fg = torch.empty_like(f)
    mk = lambda t, lo, hi: pkg.make_tensor_batch(t, dim, lo, hi)  # noqa: E731
    assert pkg.st_mul(st, None, mk(fg, 0, D), mk(f, 0, 2), mk(g, 0, 3), basis, B)
    res = torch.empty(3, B, dtype=torch.float64, device="cuda")
    assert pkg.tensor_pairing(st, None, pkg.make_scalar_batch(res[0]), mk(sig, 0, D), mk(fg, 0, D), basis, B)
    assert pkg.tensor_pairing(st, None, pkg.make_scalar_batch(res[1]), mk(sig, 0, D), mk(f, 0, 2), basis, B)
    assert pkg.tensor_pairing(st, None, pkg.make_scalar_batch(res[2]), mk(sig, 0, D), mk(g, 0, 3), basis, B)
    torch.cuda.synchronize()
    lhs, rhs = res[0].cpu().numpy(), (res[1] * res[2]).cpu().numpy()
    assert_close(lhs, rhs, 1e-11, "<S, f sh g> = <S,f><S,g>")


def test_adjoint_identities_full_size():
    """4096 tensors of W5 D5: <st_adj_mul(op, arg), x> = <arg, op sh x>,
    <left_hs_adj_lmul(x, z), y> = <z, x < y> = <left_hs_adj_rmul(z, y), x>,
    and f sh g = f < g + g < f for f, g without a degree-0 term."""
    W, D, B = 5, 5, 4096
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    gen = torch.Generator(device="cuda").manual_seed(21)
    rnd = lambda: torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=gen) - 0.5  # noqa: E731
    op, arg, x, y, z = rnd(), rnd(), rnd(), rnd(), rnd()
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    t1, t2 = torch.empty_like(x), torch.empty_like(x)
    assert pkg.st_adj_mul(st, None, full(t1), full(op), full(arg), basis, B)
    assert pkg.st_mul(st, None, full(t2), full(op), full(x), basis, B)
    torch.cuda.synchronize()
    assert_close(_pair(t1, x).cpu().numpy(), _pair(arg, t2).cpu().numpy(), 1e-11, "st_adj_mul adjoint")
    assert pkg.left_hs_mul(st, None, full(t2), full(x), full(y), basis, B)
    assert pkg.left_hs_adj_lmul(st, None, full(t1), full(x), full(z), basis, B)
    torch.cuda.synchronize()
    zxy = _pair(z, t2).cpu().numpy()
    assert_close(_pair(t1, y).cpu().numpy(), zxy, 1e-11, "left_hs_adj_lmul adjoint")
    assert pkg.left_hs_adj_rmul(st, None, full(t1), full(z), full(y), basis, B)
    torch.cuda.synchronize()
    assert_close(_pair(t1, x).cpu().numpy(), zxy, 1e-11, "left_hs_adj_rmul adjoint")
    f, g = x.clone(), y.clone()
    f[:, 0] = 0
    g[:, 0] = 0
    fg, h1, h2 = torch.empty_like(f), torch.empty_like(f), torch.empty_like(f)
    assert pkg.st_mul(st, None, full(fg), full(f), full(g), basis, B)
    assert pkg.left_hs_mul(st, None, full(h1), full(f), full(g), basis, B)
    assert pkg.left_hs_mul(st, None, full(h2), full(g), full(f), basis, B)
    torch.cuda.synchronize()
    assert_close((h1 + h2).cpu().numpy(), fg.cpu().numpy(), 1e-12, "f sh g = f < g + g < f")


def test_half_shuffle_straight_line_known_answer():
    """Along x(s) = t s e_0 the signature is exp(t e_0), and
    <exp(t e_0), e_00 < e_0> = t^3/3, <exp(t e_0), e_0 < e_00> = t^3/6
    (tests/rpp/cpu/single_thread/ops/left_hs_mul_tests.cpp:180-207)."""
    W, D, t = 2, 3, 0.7
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    db = O.degree_begin(W, D)
    sig = torch.zeros(1, dim, dtype=torch.float64, device="cuda")
    incr = torch.tensor([[t, 0.0]], dtype=torch.float64, device="cuda")
    assert pkg.signature(st, None, incr, basis, 1, length=1, out=sig)
    e0 = torch.zeros(1, dim, dtype=torch.float64, device="cuda")
    e00 = torch.zeros_like(e0)
    e0[0, db[1]] = 1.0
    e00[0, db[2]] = 1.0
    full = lambda q: pkg.make_tensor_batch(q, dim, 0, D)  # noqa: E731
    h = torch.empty_like(e0)
    res = torch.empty(2, 1, dtype=torch.float64, device="cuda")
    assert pkg.left_hs_mul(st, None, full(h), full(e00), full(e0), basis, 1)
    assert pkg.tensor_pairing(st, None, pkg.make_scalar_batch(res[0]), full(sig), full(h), basis, 1)
    torch.cuda.synchronize()
    assert abs(float(res[0, 0]) - t ** 3 / 3) <= 1e-15
    assert pkg.left_hs_mul(st, None, full(h), full(e0), full(e00), basis, 1)
    assert pkg.tensor_pairing(st, None, pkg.make_scalar_batch(res[1]), full(sig), full(h), basis, 1)
    torch.cuda.synchronize()
    assert abs(float(res[1, 0]) - t ** 3 / 6) <= 1e-15
