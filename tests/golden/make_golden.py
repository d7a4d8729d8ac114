"""Generate the golden fixtures in this directory from the reference itself.

Run in a checkout where the reference sources are available (they are compiled
from their own headers into ``oracle/_ref/librpp_ref.so`` by
``make -C oracle ref REF=<reference checkout>``):

    python tests/golden/make_golden.py

Every expected value in the fixtures is produced by the unmodified reference
CPU ``single_thread`` strategy through its public operation API; the inputs are
seeded and stored alongside, so the fixtures do not depend on a random number
generator at test time.  Files written:

* ``ops_w3d4.npz``     -- every hot-path op over the reference's degree-range cases
* ``lie_<W>_<D>.npz``  -- Hall basis tables and the t2l / l2t CSC matrices
* ``signature_w4d4.npz`` -- signatures of 8 paths of 32 steps (caller loop of ft_fmexp)
* ``kat.json``         -- reverse_index and find_bracket known answers
* ``shuffle_w3d4.npz`` -- the shuffle-algebra ops and tensor_pairing over the
  degree-range cases of the reference's shuffle tests, plus small bases
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

# Degree-range cases of tests/rpp/ft_degree_range_cases.hpp (depth four).
MUL_CASES = [
    ((0, 4), (1, 2), (1, 2)), ((0, 4), (1, 1), (2, 2)), ((0, 4), (2, 2), (1, 1)),
    ((0, 4), (0, 0), (2, 3)), ((0, 4), (2, 3), (0, 0)), ((0, 4), (0, 0), (0, 0)),
    ((0, 1), (1, 2), (1, 2)), ((3, 4), (1, 1), (1, 1)), ((0, 4), (3, 4), (2, 3)),
    ((0, 0), (1, 2), (0, 2)), ((0, 0), (0, 2), (1, 2)), ((1, 3), (1, 1), (1, 1)),
    ((0, 4), (0, 4), (0, 4)),
]
FMA_CASES = [
    ((0, 4), (0, 1), (1, 2), (1, 2)), ((0, 4), (3, 4), (1, 1), (1, 1)),
    ((0, 4), (0, 0), (2, 2), (2, 2)), ((0, 4), (1, 1), (1, 1), (2, 2)),
    ((0, 4), (1, 1), (2, 2), (1, 1)), ((0, 4), (1, 1), (0, 0), (2, 3)),
    ((0, 4), (1, 1), (2, 3), (0, 0)), ((0, 4), (0, 0), (0, 0), (0, 0)),
    ((0, 1), (2, 3), (1, 2), (1, 2)), ((3, 4), (1, 2), (1, 1), (1, 1)),
    ((0, 4), (1, 2), (3, 4), (2, 3)), ((0, 0), (1, 2), (1, 2), (0, 2)),
    ((0, 0), (1, 2), (0, 2), (1, 2)), ((0, 0), (0, 0), (1, 2), (0, 2)),
    ((1, 3), (3, 3), (1, 1), (1, 1)), ((0, 4), (0, 4), (0, 4), (0, 4)),
]
INPLACE_CASES = [
    ((0, 4), (0, 4), (0, 4)), ((1, 4), (1, 2), (1, 2)), ((2, 4), (1, 1), (0, 0)),
    ((1, 4), (0, 0), (2, 2)), ((0, 0), (0, 0), (0, 0)), ((0, 0), (1, 2), (1, 2)),
    ((0, 2), (0, 1), (3, 4)), ((3, 4), (0, 1), (0, 2)), ((0, 2), (3, 4), (3, 4)),
    ((3, 4), (0, 1), (0, 1)), ((1, 3), (1, 1), (3, 3)), ((4, 4), (0, 1), (1, 2)),
]
# tests/rpp/ft_intermediate_test_helper.hpp:25-46 (multiplier/arg ranges)
FMEXP_CASES = [
    ((0, 4), (0, 4)), ((0, 0), (0, 0)), ((1, 2), (1, 2)), ((3, 4), (1, 1)),
    ((0, 0), (3, 4)), ((3, 4), (0, 0)), ((2, 3), (3, 4)),
]
UNARY_CASES = [(0, 4), (0, 0), (1, 4), (1, 1), (1, 2), (2, 3), (3, 4), (4, 4)]
ADJ_CASES = [
    ((0, 4), (0, 4), (0, 4)), ((1, 2), (3, 3), (0, 0)), ((0, 1), (1, 1), (2, 2)),
    ((0, 1), (2, 2), (1, 1)), ((0, 0), (0, 0), (0, 0)), ((1, 3), (0, 2), (2, 4)),
    ((2, 4), (1, 1), (0, 4)),
]
ANTIPODE_CASES = [((0, 4), (0, 4)), ((1, 3), (0, 4)), ((0, 4), (2, 3)), ((2, 2), (1, 4))]


def tensor_batch(rng, n, dim, scale=1.0):
    """Dyadic inputs (multiples of 1/64 in [-1, 1]) keep the fixtures small."""
    return np.ascontiguousarray(rng.integers(-64, 65, (n, dim)) / 64.0 * scale)


def make_ops(ref: O.RefBridge, path: str) -> None:
    W, D, n = 3, 4, 2
    dim = O.tensor_dim(W, D)
    rng = np.random.default_rng(20240611)
    out = {}

    def put(name, **arrays):
        for k, v in arrays.items():
            out[f"{name}/{k}"] = np.asarray(v)

    for i, rr in enumerate(MUL_CASES):
        lhs, rhs, init = (tensor_batch(rng, n, dim) for _ in range(3))
        res = init.copy()
        ref.ft_mul(W, D, res, lhs, rhs, rr, 0.75)
        put(f"ft_mul/{i}", ranges=np.array(rr), lhs=lhs, rhs=rhs, init=init, out=res, beta=0.75)
    for i, rr in enumerate(FMA_CASES):
        a, b, c, init = (tensor_batch(rng, n, dim) for _ in range(4))
        res = init.copy()
        ref.ft_fma(W, D, res, a, b, c, rr, 0.5, -1.25)
        put(f"ft_fma/{i}", ranges=np.array(rr), a=a, b=b, c=c, init=init, out=res, alpha=0.5, beta=-1.25)
    for kind in range(3):
        for i, rr in enumerate(INPLACE_CASES):
            a, b, c = (tensor_batch(rng, n, dim) for _ in range(3))
            res = a.copy()
            ref.ft_inplace_fma(W, D, kind, res, b, c, rr, 0.5, 1.5)
            put(f"ft_inplace_fma{kind}/{i}", ranges=np.array(rr), a=a, b=b, c=c, out=res, alpha=0.5, beta=1.5)
    for i, rr in enumerate(INPLACE_CASES):
        a, b = (tensor_batch(rng, n, dim) for _ in range(2))
        res = a.copy()
        ref.ft_inplace_mul(W, D, res, b, rr[:2], -0.5)
        put(f"ft_inplace_mul/{i}", ranges=np.array(rr[:2]), a=a, b=b, out=res, beta=-0.5)
    for i, ar in enumerate(UNARY_CASES):
        for op in ("ft_exp", "ft_log"):
            arg, init = tensor_batch(rng, n, dim, 0.5), tensor_batch(rng, n, dim)
            if op == "ft_log":
                arg[:, 0] = 1.0
            res = init.copy()
            getattr(ref, op)(W, D, res, arg, ((0, D), ar))
            put(f"{op}/{i}", ranges=np.array(((0, D), ar)), arg=arg, init=init, out=res)
    for i, (mr, xr) in enumerate(FMEXP_CASES):
        mult, x, init = tensor_batch(rng, n, dim), tensor_batch(rng, n, dim, 0.5), tensor_batch(rng, n, dim)
        res = init.copy()
        rr = ((0, D), mr, xr)
        ref.ft_fmexp(W, D, res, mult, x, rr)
        put(f"ft_fmexp/{i}", ranges=np.array(rr), mult=mult, x=x, init=init, out=res)
    for left in (1, 0):
        name = "ft_adj_lmul" if left else "ft_adj_rmul"
        for i, rr in enumerate(ADJ_CASES):
            op, arg, init = (tensor_batch(rng, n, dim) for _ in range(3))
            res = init.copy()
            ref.ft_adj_mul(W, D, left, res, op, arg, rr)
            put(f"{name}/{i}", ranges=np.array(rr), op=op, arg=arg, init=init, out=res)
    for signed in (1, 0):
        name = "tensor_antipode" if signed else "tensor_reflect"
        for i, rr in enumerate(ANTIPODE_CASES):
            arg, init = tensor_batch(rng, n, dim), tensor_batch(rng, n, dim)
            res = init.copy()
            ref.antipode(W, D, signed, res, arg, rr)
            put(f"{name}/{i}", ranges=np.array(rr), arg=arg, init=init, out=res)
    np.savez_compressed(path, width=W, depth=D, **out)


# tests/rpp/cpu/single_thread/ops/st_mul_tests.cpp:222-268 (depth four):
# (out, lhs, rhs)
ST_MUL_CASES = [
    ((0, 4), (0, 4), (0, 4)), ((0, 4), (1, 4), (0, 4)), ((0, 4), (0, 4), (1, 4)),
    ((0, 4), (0, 2), (0, 4)), ((0, 4), (0, 4), (0, 2)), ((0, 4), (1, 3), (1, 2)),
    ((2, 4), (0, 4), (0, 4)), ((0, 2), (0, 4), (0, 4)), ((1, 3), (0, 2), (1, 4)),
]
# st_fma_tests.cpp:285-311 and st_inplace_fma_tests.cpp:237-262: (out, a, b, c)
ST_FMA_CASES = [
    ((0, 4), (0, 4), (0, 4), (0, 4)), ((1, 3), (1, 3), (0, 2), (2, 4)),
    ((1, 3), (1, 3), (1, 2), (1, 4)), ((0, 4), (2, 2), (0, 0), (0, 1)),
]
ST_INPLACE_CASES = [((0, 4), (0, 4), (0, 4)), ((1, 3), (1, 2), (1, 4)), ((1, 4), (0, 2), (1, 4)),
                    ((0, 0), (0, 1), (0, 2))]
# tests/rpp/shuffle_adjoint_test_helper.hpp:20-36 (out, op, arg) and the two
# extra half-shuffle cases of half_shuffle_adjoint_test_helper.hpp:84-106.
SH_ADJ_CASES = [
    ((0, 4), (0, 4), (0, 4)), ((0, 4), (0, 0), (1, 2)), ((0, 4), (1, 2), (2, 3)),
    ((0, 4), (1, 1), (3, 3)), ((0, 4), (3, 4), (0, 2)), ((0, 1), (0, 1), (3, 4)),
    ((3, 4), (1, 2), (1, 2)), ((0, 4), (0, 0), (0, 0)), ((0, 4), (1, 2), (0, 0)),
    ((0, 0), (2, 2), (2, 2)), ((0, 0), (1, 1), (2, 2)), ((1, 3), (0, 1), (2, 3)),
    ((4, 4), (0, 0), (4, 4)),
]
HS_ADJ_EXTRA = [((1, 2), (1, 2), (2, 4)), ((0, 4), (0, 4), (0, 0))]
# left_hs_mul_tests.cpp:136: every (lhs, rhs) pair of these ranges with the
# full output, and every output range with full operands.
HS_RANGES = [(0, 0), (0, 1), (1, 2), (2, 4), (0, 4)]
PAIRING_CASES = [((0, 4), (0, 4)), ((1, 3), (0, 4)), ((0, 1), (2, 4)), ((2, 2), (2, 3)), ((4, 4), (0, 4))]


def make_shuffle(ref: O.RefBridge, path: str) -> None:
    """Inputs are stored once per basis; every case stores its ranges and the
    reference's output, computed from `init` (NaN-free dyadic values)."""
    rng = np.random.default_rng(31337)
    out = {}
    n = 2

    def put(name, **arrays):
        for k, v in arrays.items():
            out[f"{name}/{k}"] = np.asarray(v)

    W, D = 3, 4
    dim = O.tensor_dim(W, D)
    x, y, z, init = (tensor_batch(rng, n, dim) for _ in range(4))
    out.update({"inputs/x": x, "inputs/y": y, "inputs/z": z, "inputs/init": init})
    for i, rr in enumerate(ST_MUL_CASES):
        res = init.copy()
        ref.st_mul(W, D, res, x, y, rr, 0.75)
        put(f"st_mul/{i}", ranges=np.array(rr), out=res, beta=0.75)
    for i, rr in enumerate(ST_FMA_CASES):
        res = init.copy()
        ref.st_fma(W, D, res, z, x, y, rr, 0.5, -1.25)
        put(f"st_fma/{i}", ranges=np.array(rr), out=res, alpha=0.5, beta=-1.25)
    for i, rr in enumerate(ST_INPLACE_CASES):
        res = z.copy()
        ref.st_inplace_fma(W, D, res, x, y, rr, 0.5, 1.5)
        put(f"st_inplace_fma/{i}", ranges=np.array(rr), out=res, alpha=0.5, beta=1.5)
    hs = [((0, 4), l, r) for l in HS_RANGES for r in HS_RANGES] + [(o, (0, 4), (0, 4)) for o in HS_RANGES]
    for i, rr in enumerate(hs):
        res = init.copy()
        ref.left_hs_mul(W, D, res, x, y, rr, 3.0)
        put(f"left_hs_mul/{i}", ranges=np.array(rr), out=res, beta=3.0)
    for i, rr in enumerate(SH_ADJ_CASES):
        res = init.copy()
        ref.st_adj_mul(W, D, res, x, y, rr)
        put(f"st_adj_mul/{i}", ranges=np.array(rr), out=res)
    for lmul in (1, 0):
        name = "left_hs_adj_lmul" if lmul else "left_hs_adj_rmul"
        for i, rr in enumerate(SH_ADJ_CASES + HS_ADJ_EXTRA):
            # rr = (out, fixed operand, cotangent); the operator takes
            # (integrator, integrand) = (fixed, cotangent) for lmul and
            # (cotangent, fixed) for rmul.
            res = init.copy()
            if lmul:
                ref.left_hs_adjoint(W, D, 1, res, x, y, (rr[0], rr[1], rr[2]))
            else:
                ref.left_hs_adjoint(W, D, 0, res, y, x, (rr[0], rr[2], rr[1]))
            put(f"{name}/{i}", ranges=np.array(rr), out=res)
    for i, fr in enumerate(PAIRING_CASES):
        put(f"tensor_pairing/{i}", ranges=np.array(fr), out=ref.tensor_pairing(W, D, x, y, fr))
    # the small bases of half_shuffle_adjoint_tests (width, depth): full views
    for W2, D2 in [(1, 4), (2, 2), (4, 0)]:
        dim2 = O.tensor_dim(W2, D2)
        a, b, c = (tensor_batch(rng, n, dim2) for _ in range(3))
        full = (0, D2)
        key = f"small_{W2}_{D2}"
        out[f"{key}/a"], out[f"{key}/b"], out[f"{key}/init"] = a, b, c
        for name in ("st_mul", "left_hs_mul", "st_adj_mul", "left_hs_adj_lmul", "left_hs_adj_rmul"):
            res = c.copy()
            if name == "st_mul":
                ref.st_mul(W2, D2, res, a, b, (full, full, full))
            elif name == "left_hs_mul":
                ref.left_hs_mul(W2, D2, res, a, b, (full, full, full))
            elif name == "st_adj_mul":
                ref.st_adj_mul(W2, D2, res, a, b, (full, full, full))
            else:
                ref.left_hs_adjoint(W2, D2, name.endswith("lmul"), res, a, b, (full, full, full))
            out[f"{key}/{name}"] = res
    np.savez_compressed(path, width=3, depth=4, **out)


def make_lie(ref: O.RefBridge, W: int, D: int, path: str, with_spmv: bool) -> None:
    db, pairs = ref.hall_basis(W, D)
    t2l = ref.conversion_matrix(W, D, "t2l")
    l2t = ref.conversion_matrix(W, D, "l2t")
    arrays = dict(width=W, depth=D, degree_begin=db, pairs=pairs,
                  t2l_offsets=t2l[0], t2l_indices=t2l[1], t2l_values=t2l[2], t2l_dims=np.array(t2l[3]),
                  l2t_offsets=l2t[0], l2t_indices=l2t[1], l2t_values=l2t[2], l2t_dims=np.array(l2t[3]))
    if with_spmv:
        rng = np.random.default_rng(7 + W * 100 + D)
        n, dim, lie = 4, O.tensor_dim(W, D), int(db[-1])
        tens = rng.uniform(-1, 1, (n, dim))
        lie_out = np.full((n, lie), np.nan)
        ref.tensor_lie(W, D, True, t2l, lie_out, tens)
        lie_in = rng.uniform(-1, 1, (n, lie))
        tens_out = np.full((n, dim), np.nan)
        ref.tensor_lie(W, D, False, l2t, tens_out, lie_in)
        arrays.update(t2l_arg=tens, t2l_out=lie_out, l2t_arg=lie_in, l2t_out=tens_out)
    np.savez_compressed(path, **arrays)


def make_signature(ref: O.RefBridge, path: str) -> None:
    W, D, B, L = 4, 4, 8, 32
    rng = np.random.default_rng(99)
    incr = rng.normal(0.0, 1.0 / np.sqrt(L), (B * L, W))
    offsets = np.arange(B + 1, dtype=np.int64) * L
    sig, _ = ref.signature(W, D, incr, offsets)
    np.savez_compressed(path, width=W, depth=D, incr=incr, offsets=offsets, sig=sig)


def make_kat(ref: O.RefBridge, path: str) -> None:
    kat = {"reverse_index": [], "find_bracket": []}
    for W, deg, idx in [(3, 4, 5), (3, 4, 80), (5, 5, 1234), (2, 12, 3000), (16, 3, 4000), (4, 1, 3), (4, 0, 0)]:
        kat["reverse_index"].append([W, deg, idx, int(ref.reverse_index(W, deg, idx))])
    for W, D, l, r, h in [(3, 4, 1, 2, 2), (3, 4, 1, 2, 0), (3, 4, 2, 5, 3), (3, 4, 3, 4, 3), (3, 4, 2, 1, 2),
                          (3, 4, 1, 1, 2), (3, 4, 1, 6, 3), (3, 4, 1, 9, 4), (5, 5, 3, 100, 0)]:
        kat["find_bracket"].append([W, D, l, r, h, int(ref.find_bracket(W, D, l, r, h))])
    with open(path, "w") as f:
        json.dump(kat, f, indent=1)


def main() -> None:
    ref = O.RefBridge()
    make_ops(ref, os.path.join(HERE, "ops_w3d4.npz"))
    for W, D in [(3, 4), (4, 4), (5, 5), (2, 6)]:
        make_lie(ref, W, D, os.path.join(HERE, f"lie_{W}_{D}.npz"), with_spmv=(W, D) in [(3, 4), (5, 5)])
    make_signature(ref, os.path.join(HERE, "signature_w4d4.npz"))
    make_kat(ref, os.path.join(HERE, "kat.json"))
    make_shuffle(ref, os.path.join(HERE, "shuffle_w3d4.npz"))


if __name__ == "__main__":
    main()
