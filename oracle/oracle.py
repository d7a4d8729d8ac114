"""Python bindings of the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  The library in the
package directory never imports it.

* ``Oracle`` wraps ``_build/librpp_oracle.so`` (the plain-C restatement in
  ``rpp_oracle.c``; FP64 throughout).
* ``lie_tables`` restates, in pure Python, the reference's Hall basis
  (include/rpp/basis/hall_basis.hpp:35-88), its bracket-expansion cache
  (include/rpp/basis/lie_multiplication.hpp:163-251) and the sparse conversion
  builders ``make_t2l_matrix`` (include/rpp/sparse/t2l_matrix.hpp:57-142) and
  ``make_l2t_matrix`` (include/rpp/sparse/l2t_matrix.hpp:58-114).  Integer
  tables must match the reference bit for bit; the golden fixtures pin them.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librpp_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "librpp_ref.so")


class Arg(ctypes.Structure):
    """Mirror of ``orc_arg``: one operand batch (data, stride, degree range)."""

    _fields_ = [
        ("data", ctypes.c_void_p),
        ("stride", ctypes.c_int64),
        ("min_degree", ctypes.c_int32),
        ("max_degree", ctypes.c_int32),
    ]


def build(ref: bool = False) -> None:
    """Compile the oracle (and, when asked and present, the reference bridge)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def tensor_dim(width: int, depth: int) -> int:
    """Dimension of T^(depth)(R^width), degree 0 included
    (include/rpp/basis/tensor_basis.hpp:122-130)."""
    dim, p = 0, 1
    for _ in range(depth + 1):
        dim += p
        p *= width
    return dim


def degree_begin(width: int, depth: int) -> list[int]:
    """degree_begin[n] = (W^n - 1)/(W - 1); depth + 2 entries."""
    out, p = [0], 1
    for _ in range(depth + 1):
        out.append(out[-1] + p)
        p *= width
    return out


def _arg(a: np.ndarray | None, stride: int, rng: tuple[int, int]) -> Arg | None:
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return Arg(a.ctypes.data, stride, rng[0], rng[1])


class Oracle:
    """ctypes front of the plain-C oracle.  Arrays are float64 [batch, stride]."""

    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            build()
        self.lib = ctypes.CDLL(path)
        P = ctypes.POINTER(Arg)
        i32, i64, dbl = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
        L = self.lib
        L.orc_ft_fma.argtypes = [i32, i32, i64, P, P, P, P, dbl, dbl]
        L.orc_ft_inplace_fma.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P, dbl, dbl]
        L.orc_ft_inplace_mul.argtypes = [i32, i32, i64, P, P, dbl]
        L.orc_ft_exp.argtypes = [i32, i32, i64, P, P]
        L.orc_ft_fmexp.argtypes = [i32, i32, i64, P, P, P]
        L.orc_ft_log.argtypes = [i32, i32, i64, P, P]
        L.orc_ft_adjoint.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P]
        L.orc_antipode.argtypes = [i32, i32, i64, ctypes.c_int, P, P]
        L.orc_reverse_index.argtypes = [i32, i32, i64]
        L.orc_reverse_index.restype = i64
        vp = ctypes.c_void_p
        L.orc_spmv.argtypes = [i64, ctypes.c_int, i64, vp, vp, vp, vp, i64, i64, i64, vp, i64, i64, dbl]
        L.orc_signature.argtypes = [i32, i32, i64, vp, vp, vp, vp, vp, i32]
        L.orc_st.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P, P, dbl, dbl]
        L.orc_left_hs_mul.argtypes = [i32, i32, i64, P, P, P, dbl]
        L.orc_st_adj_mul.argtypes = [i32, i32, i64, P, P, P]
        L.orc_left_hs_adjoint.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P, dbl]
        L.orc_tensor_pairing.argtypes = [i32, i32, i64, vp, P, P]

    @staticmethod
    def _p(x):
        return None if x is None else ctypes.byref(x)

    def ft_mul(self, W, D, out, lhs, rhs, ranges, beta=1.0):
        """out = beta * lhs (x) rhs.  ranges = (out, lhs, rhs) degree ranges."""
        n, s = out.shape
        self.lib.orc_ft_fma(W, D, n, self._p(_arg(out, s, ranges[0])), None,
                            self._p(_arg(lhs, s, ranges[1])), self._p(_arg(rhs, s, ranges[2])),
                            0.0, beta)

    def ft_fma(self, W, D, out, a, b, c, ranges, alpha=1.0, beta=1.0):
        n, s = out.shape
        self.lib.orc_ft_fma(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(a, s, ranges[1])),
                            self._p(_arg(b, s, ranges[2])), self._p(_arg(c, s, ranges[3])), alpha, beta)

    def ft_inplace_fma(self, W, D, kind, a, b, c, ranges, alpha=1.0, beta=1.0):
        n, s = a.shape
        self.lib.orc_ft_inplace_fma(W, D, n, kind, self._p(_arg(a, s, ranges[0])),
                                    self._p(_arg(b, s, ranges[1])), self._p(_arg(c, s, ranges[2])),
                                    alpha, beta)

    def ft_inplace_mul(self, W, D, lhs, rhs, ranges, beta=1.0):
        n, s = lhs.shape
        self.lib.orc_ft_inplace_mul(W, D, n, self._p(_arg(lhs, s, ranges[0])),
                                    self._p(_arg(rhs, s, ranges[1])), beta)

    def ft_exp(self, W, D, out, arg, ranges):
        n, s = out.shape
        self.lib.orc_ft_exp(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(arg, s, ranges[1])))

    def ft_fmexp(self, W, D, out, mult, x, ranges):
        n, s = out.shape
        self.lib.orc_ft_fmexp(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(mult, s, ranges[1])),
                              self._p(_arg(x, s, ranges[2])))

    def ft_log(self, W, D, out, arg, ranges):
        n, s = out.shape
        self.lib.orc_ft_log(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(arg, s, ranges[1])))

    def ft_adj_mul(self, W, D, left, out, op, arg, ranges):
        n, s = out.shape
        self.lib.orc_ft_adjoint(W, D, n, int(left), self._p(_arg(out, s, ranges[0])),
                                self._p(_arg(op, s, ranges[1])), self._p(_arg(arg, s, ranges[2])))

    def antipode(self, W, D, signed, out, arg, ranges):
        n, s = out.shape
        self.lib.orc_antipode(W, D, n, int(signed), self._p(_arg(out, s, ranges[0])),
                              self._p(_arg(arg, s, ranges[1])))

    def reverse_index(self, W, degree, idx):
        return self.lib.orc_reverse_index(W, degree, idx)

    def spmv(self, csc, offsets, indices, values, out, out_begin, out_len, arg, arg_begin, alpha=1.0):
        """Batched SpMV with begin-relative indexing (CPU strategy semantics)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        indices = np.ascontiguousarray(indices, dtype=np.int64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        n = out.shape[0]
        self.lib.orc_spmv(n, int(csc), len(offsets) - 1, offsets.ctypes.data, indices.ctypes.data,
                          values.ctypes.data, out.ctypes.data, out.shape[1], out_begin, out_len,
                          arg.ctypes.data, arg.shape[1], arg_begin, alpha)

    def signature(self, W, D, incr, offsets, ell=None, want_sig=True, threads=1):
        """Signatures (and, with ell, gradients of sum_b <ell_b, S(x_b)>) of a
        ragged batch.  incr: float64 [total_steps, W]; offsets: int64 [B + 1]."""
        incr = np.ascontiguousarray(incr, dtype=np.float64)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        B = len(offsets) - 1
        dim = tensor_dim(W, D)
        sig = np.zeros((B, dim)) if want_sig else None
        grad = np.zeros_like(incr) if ell is not None else None
        if ell is not None:
            ell = np.ascontiguousarray(ell, dtype=np.float64)
        self.lib.orc_signature(W, D, B, incr.ctypes.data, offsets.ctypes.data,
                               None if sig is None else sig.ctypes.data,
                               None if ell is None else ell.ctypes.data,
                               None if grad is None else grad.ctypes.data, threads)
        return sig, grad



    # -- shuffle algebra -------------------------------------------------
    def _st(self, W, D, mode, out, a, b, c, ranges, alpha, beta):
        n, s = out.shape
        return self.lib.orc_st(W, D, n, mode, self._p(_arg(out, s, ranges[0])), self._p(_arg(a, s, ranges[1])),
                               self._p(_arg(b, s, ranges[2])), self._p(_arg(c, s, ranges[3])), alpha, beta)

    def st_mul(self, W, D, out, lhs, rhs, ranges, beta=1.0):
        """out = beta * lhs sh rhs.  ranges = (out, lhs, rhs)."""
        self._st(W, D, 0, out, None, lhs, rhs, (ranges[0], (1, 0), ranges[1], ranges[2]), 0.0, beta)

    def st_fma(self, W, D, out, a, b, c, ranges, alpha=1.0, beta=1.0):
        """out = alpha*a + beta * b sh c.  ranges = (out, a, b, c)."""
        self._st(W, D, 1, out, a, b, c, ranges, alpha, beta)

    def st_inplace_fma(self, W, D, a, b, c, ranges, alpha=1.0, beta=1.0):
        """a = alpha*a + beta * b sh c.  ranges = (a, b, c)."""
        self._st(W, D, 2, a, None, b, c, (ranges[0], (1, 0), ranges[1], ranges[2]), alpha, beta)

    def left_hs_mul(self, W, D, out, integrator, integrand, ranges, beta=1.0):
        n, s = out.shape
        self.lib.orc_left_hs_mul(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(integrator, s, ranges[1])),
                                 self._p(_arg(integrand, s, ranges[2])), beta)

    def st_adj_mul(self, W, D, out, op, arg, ranges):
        n, s = out.shape
        self.lib.orc_st_adj_mul(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(op, s, ranges[1])),
                                self._p(_arg(arg, s, ranges[2])))

    def left_hs_adjoint(self, W, D, lmul, out, integrator, integrand, ranges, beta=1.0):
        """lmul: (out, fixed integrator, integrand cotangent); rmul: (out,
        integrator cotangent, fixed integrand) -- the reference operator's order."""
        n, s = out.shape
        self.lib.orc_left_hs_adjoint(W, D, n, int(lmul), self._p(_arg(out, s, ranges[0])),
                                     self._p(_arg(integrator, s, ranges[1])),
                                     self._p(_arg(integrand, s, ranges[2])), beta)

    def tensor_pairing(self, W, D, functional, arg, ranges):
        n, s = functional.shape
        res = np.zeros(n)
        self.lib.orc_tensor_pairing(W, D, n, res.ctypes.data, self._p(_arg(functional, s, ranges[0])),
                                    self._p(_arg(arg, s, ranges[1])))
        return res

# ---------------------------------------------------------------------------
# Hall basis, bracket expansions and the tensor <-> Lie conversion matrices.
# ---------------------------------------------------------------------------

def hall_basis(width: int, depth: int):
    """Hall set as (degree_begin, pairs).  Key 0 is the (0, 0) sentinel, keys
    1..W are the letters (0, letter); higher keys are (left, right) pairs with
    left < right and left >= the left parent of right, degree by degree,
    left degree ascending (include/rpp/basis/hall_basis.hpp:35-88)."""
    pairs = [(0, 0)]
    db = [0, 1]
    if depth > 0:
        for letter in range(1, width + 1):
            pairs.append((0, letter))
        db.append(1 + width)
        for degree in range(2, depth + 1):
            for ld in range(1, degree // 2 + 1):
                rd = degree - ld
                for left in range(db[ld], db[ld + 1]):
                    for right in range(max(left + 1, db[rd]), db[rd + 1]):
                        if pairs[right][0] <= left:
                            pairs.append((left, right))
            db.append(len(pairs))
    return db, pairs


class LieTables:
    """Bracket expansions in the Hall basis, restating the reference's
    LieMultiplicationCache (include/rpp/basis/lie_multiplication.hpp:163-251),
    with exact integer coefficients."""

    def __init__(self, width: int, depth: int):
        self.width, self.depth = width, depth
        self.db, self.pairs = hall_basis(width, depth)
        self.true_size = self.db[-1]
        self.key_of = {p: k for k, p in enumerate(self.pairs) if k > 0}
        self._deg = {}
        for d in range(len(self.db) - 1):
            for k in range(self.db[d], self.db[d + 1]):
                self._deg[k] = d
        self.cache: dict[tuple[int, int], list[tuple[int, int]]] = {}

    def degree(self, key: int) -> int:
        return self._deg[key]

    def find_bracket(self, left: int, right: int) -> int:
        """Key of the Hall element (left, right), or 0 if there is none
        (include/rpp/basis/lie_basis.hpp:105-148)."""
        return self.key_of.get((left, right), 0)

    def bracket(self, left: int, right: int) -> list[tuple[int, int]]:
        """[left, right] as a sorted list of (key, coefficient)."""
        if left <= 0 or right <= 0 or left == right:
            return []
        if left >= self.true_size or right >= self.true_size:
            return []
        if self.degree(left) + self.degree(right) > self.depth:
            return []
        hit = self.cache.get((left, right))
        if hit is not None:
            return hit
        k = self.find_bracket(left, right)
        if k:
            res = [(k, 1)]
        else:
            k = self.find_bracket(right, left)
            if k:
                res = [(k, -1)]
            elif right < left:
                res = [(key, -c) for key, c in self.bracket(right, left)]
            else:
                # Jacobi: [l, [a, b]] = [[l, a], b] - [[l, b], a]
                acc: dict[int, int] = {}
                a, b = self.pairs[right]
                if a > 0 and a != left:
                    for ok, ov in self.bracket(left, a):
                        for ik, iv in self.bracket(ok, b):
                            acc[ik] = acc.get(ik, 0) + ov * iv
                if b != left:
                    for ok, ov in self.bracket(left, b):
                        for ik, iv in self.bracket(ok, a):
                            acc[ik] = acc.get(ik, 0) - ov * iv
                res = sorted((kk, v) for kk, v in acc.items() if v != 0)
        self.cache[(left, right)] = res
        return res

    def t2l_csc(self):
        """make_t2l_matrix: CSC, outer = tensor index (degree 0 included),
        inner = Lie index (key - 1).  Column of word w = (1/|w|) * the
        right-normed bracket [w1, [w2, ... wn]] expanded in the Hall basis
        (include/rpp/sparse/t2l_matrix.hpp:57-142)."""
        W, D = self.width, self.depth
        cols: list[dict[int, Fraction]] = [{}]  # empty word
        if D > 0:
            for i in range(W):
                cols.append({i: Fraction(1)})
        offset, prev = 1, W
        for degree in range(2, D + 1):
            size = prev * W
            for i in range(size):
                lparent = 1 + i // prev
                rparent = offset + i % prev
                frame: dict[int, Fraction] = {}
                if lparent != rparent:
                    lval = cols[lparent][lparent - 1]
                    for ridx, rval in sorted(cols[rparent].items()):
                        for key, c in self.bracket(lparent, 1 + ridx):
                            frame[key - 1] = frame.get(key - 1, Fraction(0)) + c * lval * rval
                cols.append({k: v for k, v in frame.items() if v != 0})
            offset = 1 + offset * W
            prev = size
        # normalise by degree; the divisions run in floating point in the
        # reference (value * (1/degree)), reproduced when the values are emitted.
        return self._emit(cols, normalise=True)

    def l2t_csc(self):
        """make_l2t_matrix: CSC, outer = Lie index (key - 1), inner = tensor
        index; the column of a Hall element is its commutator expansion
        (include/rpp/sparse/l2t_matrix.hpp:21-114)."""
        W, D = self.width, self.depth
        frames: list[dict[int, int]] = []
        if D > 0:
            for letter in range(1, W + 1):
                frames.append({letter: 1})
        for d in range(2, D + 1):
            for key in range(self.db[d], self.db[d + 1]):
                left, right = self.pairs[key]
                lf, rf = frames[left - 1], frames[right - 1]
                lo = W ** self.degree(left)
                ro = W ** self.degree(right)
                acc: dict[int, int] = {}
                for li, lv in lf.items():
                    for ri, rv in rf.items():
                        acc[li * ro + ri] = acc.get(li * ro + ri, 0) + lv * rv
                        acc[ri * lo + li] = acc.get(ri * lo + li, 0) - rv * lv
                frames.append({k: v for k, v in acc.items() if v != 0})
        offsets, indices, values = [0], [], []
        for f in frames:
            for k in sorted(f):
                indices.append(k)
                values.append(float(f[k]))
            offsets.append(len(indices))
        return (np.array(offsets, np.int64), np.array(indices, np.int64), np.array(values),
                (len(frames), tensor_dim(W, D)))

    def _emit(self, cols, normalise):
        W, D = self.width, self.depth
        offsets, indices, values = [0], [], []
        deg_of_col = []
        for d in range(D + 1):
            deg_of_col += [d] * (W ** d)
        for c, col in enumerate(cols):
            d = deg_of_col[c]
            for k in sorted(col):
                v = float(col[k])
                if normalise and d >= 2:
                    v = v * (1.0 / d)
                indices.append(k)
                values.append(v)
            offsets.append(len(indices))
        return (np.array(offsets, np.int64), np.array(indices, np.int64), np.array(values),
                (len(cols), self.true_size - 1))


def csc_to_csr(offsets, indices, values, outer_dim, inner_dim):
    """Transpose a compressed matrix (the reference's swap_format,
    include/rpp/sparse/detail/compressed_matrix.hpp:675-744): entries of each
    new outer slot keep ascending old-outer order."""
    counts = np.bincount(indices, minlength=inner_dim)
    new_off = np.zeros(inner_dim + 1, np.int64)
    np.cumsum(counts, out=new_off[1:])
    new_idx = np.empty_like(indices)
    new_val = np.empty_like(values)
    pos = new_off[:-1].copy()
    for o in range(outer_dim):
        for e in range(offsets[o], offsets[o + 1]):
            r = indices[e]
            new_idx[pos[r]] = o
            new_val[pos[r]] = values[e]
            pos[r] += 1
    return new_off, new_idx, new_val


class RefBridge(Oracle):
    """Same interface as ``Oracle`` but backed by ``_ref/librpp_ref.so``, the
    unmodified reference CPU strategy compiled from its headers (built only
    where the reference checkout exists; used to pin the oracle and to write the
    golden fixtures)."""

    def __init__(self, path: str = REF_LIB_PATH):
        if not os.path.exists(path):
            build(ref=True)
        self.lib = ctypes.CDLL(path)
        P = ctypes.POINTER(Arg)
        i32, i64, dbl, vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
        L = self.lib
        L.ref_ft_mul.argtypes = [i32, i32, i64, P, P, P, dbl]
        L.ref_ft_fma.argtypes = [i32, i32, i64, P, P, P, P, dbl, dbl]
        L.ref_ft_inplace_fma.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P, dbl, dbl]
        L.ref_ft_inplace_mul.argtypes = [i32, i32, i64, P, P, dbl]
        L.ref_ft_exp.argtypes = [i32, i32, i64, P, P]
        L.ref_ft_fmexp.argtypes = [i32, i32, i64, P, P, P]
        L.ref_ft_log.argtypes = [i32, i32, i64, P, P]
        L.ref_ft_adjoint.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P]
        L.ref_antipode.argtypes = [i32, i32, i64, ctypes.c_int, P, P]
        L.ref_reverse_index.argtypes = [i32, i32, i32, i64]
        L.ref_reverse_index.restype = i64
        L.ref_hall_basis.argtypes = [i32, i32, vp, vp, i64]
        L.ref_hall_basis.restype = i64
        L.ref_find_bracket.argtypes = [i32, i32, i64, i64, i32]
        L.ref_find_bracket.restype = i64
        L.ref_conversion_matrix.argtypes = [i32, i32, ctypes.c_int, vp, i64, vp, vp, i64, vp]
        L.ref_conversion_matrix.restype = i64
        L.ref_tensor_lie.argtypes = [i32, i32, i64, ctypes.c_int, i64, i64, i64, vp, vp, vp, vp, i64, vp, i64]
        L.ref_signature.argtypes = [i32, i32, i64, vp, vp, vp, i32]
        L.ref_signature_grad.argtypes = [i32, i32, i64, vp, vp, vp, vp, vp, i32]
        L.ref_st.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P, P, dbl, dbl]
        L.ref_st_adj_mul.argtypes = [i32, i32, i64, P, P, P]
        L.ref_left_hs_mul.argtypes = [i32, i32, i64, P, P, P, dbl]
        L.ref_left_hs_adjoint.argtypes = [i32, i32, i64, ctypes.c_int, P, P, P]
        L.ref_tensor_pairing.argtypes = [i32, i32, i64, vp, P, P]

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError(f"reference op failed with status {rc}")

    def ft_mul(self, W, D, out, lhs, rhs, ranges, beta=1.0):
        n, s = out.shape
        self._chk(self.lib.ref_ft_mul(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(lhs, s, ranges[1])),
                                      self._p(_arg(rhs, s, ranges[2])), beta))

    def ft_fma(self, W, D, out, a, b, c, ranges, alpha=1.0, beta=1.0):
        n, s = out.shape
        self._chk(self.lib.ref_ft_fma(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(a, s, ranges[1])),
                                      self._p(_arg(b, s, ranges[2])), self._p(_arg(c, s, ranges[3])), alpha, beta))

    def ft_inplace_fma(self, W, D, kind, a, b, c, ranges, alpha=1.0, beta=1.0):
        n, s = a.shape
        self._chk(self.lib.ref_ft_inplace_fma(W, D, n, kind, self._p(_arg(a, s, ranges[0])),
                                              self._p(_arg(b, s, ranges[1])), self._p(_arg(c, s, ranges[2])),
                                              alpha, beta))

    def ft_inplace_mul(self, W, D, lhs, rhs, ranges, beta=1.0):
        n, s = lhs.shape
        self._chk(self.lib.ref_ft_inplace_mul(W, D, n, self._p(_arg(lhs, s, ranges[0])),
                                              self._p(_arg(rhs, s, ranges[1])), beta))

    def ft_exp(self, W, D, out, arg, ranges):
        n, s = out.shape
        self._chk(self.lib.ref_ft_exp(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(arg, s, ranges[1]))))

    def ft_fmexp(self, W, D, out, mult, x, ranges):
        n, s = out.shape
        self._chk(self.lib.ref_ft_fmexp(W, D, n, self._p(_arg(out, s, ranges[0])),
                                        self._p(_arg(mult, s, ranges[1])), self._p(_arg(x, s, ranges[2]))))

    def ft_log(self, W, D, out, arg, ranges):
        n, s = out.shape
        self._chk(self.lib.ref_ft_log(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(arg, s, ranges[1]))))

    def ft_adj_mul(self, W, D, left, out, op, arg, ranges):
        n, s = out.shape
        self._chk(self.lib.ref_ft_adjoint(W, D, n, int(left), self._p(_arg(out, s, ranges[0])),
                                          self._p(_arg(op, s, ranges[1])), self._p(_arg(arg, s, ranges[2]))))

    def antipode(self, W, D, signed, out, arg, ranges):
        n, s = out.shape
        self._chk(self.lib.ref_antipode(W, D, n, int(signed), self._p(_arg(out, s, ranges[0])),
                                        self._p(_arg(arg, s, ranges[1]))))

    def reverse_index(self, W, degree, idx):
        return self.lib.ref_reverse_index(W, max(degree, 1), degree, idx)

    def hall_basis(self, W, D):
        db = np.zeros(D + 2, np.int64)
        cap = 1 << 22
        pairs = np.zeros(cap, np.int64)
        ts = self.lib.ref_hall_basis(W, D, db.ctypes.data, pairs.ctypes.data, cap)
        assert ts >= 0
        return db, pairs[: 2 * ts].reshape(ts, 2)

    def find_bracket(self, W, D, left, right, hint=0):
        return self.lib.ref_find_bracket(W, D, left, right, hint)

    def conversion_matrix(self, W, D, which):
        """which = 't2l' or 'l2t'; returns (offsets, indices, values, (outer, inner))."""
        cap = 1 << 23
        off = np.zeros(cap, np.int64)
        idx = np.zeros(cap, np.int64)
        val = np.zeros(cap)
        dims = np.zeros(3, np.int64)
        nnz = self.lib.ref_conversion_matrix(W, D, 0 if which == "t2l" else 1, off.ctypes.data, cap,
                                             idx.ctypes.data, val.ctypes.data, cap, dims.ctypes.data)
        assert nnz >= 0
        outer = int(dims[1])
        return off[: outer + 1].copy(), idx[:nnz].copy(), val[:nnz].copy(), (outer, int(dims[2]))

    def tensor_lie(self, W, D, to_lie, csc, out, arg):
        off, idx, val, (outer, inner) = csc
        n = out.shape[0]
        self._chk(self.lib.ref_tensor_lie(W, D, n, int(to_lie), len(idx), outer, inner, off.ctypes.data,
                                          idx.ctypes.data, val.ctypes.data, out.ctypes.data, out.shape[1],
                                          arg.ctypes.data, arg.shape[1]))

    def signature(self, W, D, incr, offsets, ell=None, want_sig=True, threads=1):
        """Forward: the caller loop of ft_fmexp.  With ell, also the gradient of
        sum_b <ell_b, S(x_b)> by the stored-prefix reverse pass composed from
        the reference's ft_exp, ft_adj_lmul and ft_adj_rmul."""
        incr = np.ascontiguousarray(incr, dtype=np.float64)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        B = len(offsets) - 1
        sig = np.zeros((B, tensor_dim(W, D))) if want_sig or ell is None else None
        if ell is None:
            self._chk(self.lib.ref_signature(W, D, B, incr.ctypes.data, offsets.ctypes.data, sig.ctypes.data,
                                             threads))
            return sig, None
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        grad = np.zeros_like(incr)
        self._chk(self.lib.ref_signature_grad(W, D, B, incr.ctypes.data, offsets.ctypes.data, ell.ctypes.data,
                                              None if sig is None else sig.ctypes.data, grad.ctypes.data, threads))
        return sig, grad

    def _st(self, W, D, mode, out, a, b, c, ranges, alpha, beta):
        n, s = out.shape
        self._chk(self.lib.ref_st(W, D, n, mode, self._p(_arg(out, s, ranges[0])), self._p(_arg(a, s, ranges[1])),
                                  self._p(_arg(b, s, ranges[2])), self._p(_arg(c, s, ranges[3])), alpha, beta))

    def left_hs_mul(self, W, D, out, integrator, integrand, ranges, beta=1.0):
        n, s = out.shape
        self._chk(self.lib.ref_left_hs_mul(W, D, n, self._p(_arg(out, s, ranges[0])),
                                           self._p(_arg(integrator, s, ranges[1])),
                                           self._p(_arg(integrand, s, ranges[2])), beta))

    def st_adj_mul(self, W, D, out, op, arg, ranges):
        n, s = out.shape
        self._chk(self.lib.ref_st_adj_mul(W, D, n, self._p(_arg(out, s, ranges[0])), self._p(_arg(op, s, ranges[1])),
                                          self._p(_arg(arg, s, ranges[2]))))

    def left_hs_adjoint(self, W, D, lmul, out, integrator, integrand, ranges, beta=1.0):
        """The reference's CPU operators take no scale factor: beta must be 1."""
        assert beta == 1.0
        n, s = out.shape
        self._chk(self.lib.ref_left_hs_adjoint(W, D, n, int(lmul), self._p(_arg(out, s, ranges[0])),
                                               self._p(_arg(integrator, s, ranges[1])),
                                               self._p(_arg(integrand, s, ranges[2]))))

    def tensor_pairing(self, W, D, functional, arg, ranges):
        n, s = functional.shape
        res = np.full(n, np.nan)
        self._chk(self.lib.ref_tensor_pairing(W, D, n, res.ctypes.data, self._p(_arg(functional, s, ranges[0])),
                                              self._p(_arg(arg, s, ranges[1]))))
        return res
