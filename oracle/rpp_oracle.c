/*
 * rpp_oracle.c -- CPU oracle for the batched free-tensor path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to produce the
 * expected values.  Nothing in the shipped library links, loads or calls it.
 *
 * It restates, in plain C99 and in FP64, the semantics of RoughPathPrimitives'
 * CPU `single_thread` strategy for the operations on the hot path.  Every
 * function cites the reference file:line whose behaviour it follows (paths are
 * relative to the reference project's root).  Accumulation order follows the
 * word-split definition used by the reference's own test references
 * (tests/rpp/cpu/single_thread/ops/cpu_typed_ft_ops_test_helper.hpp:160-259),
 * not the CPU tiler, so values agree with the reference to rounding (1e-12
 * relative with a floor of one, the reference's own tolerance), while every
 * index computation is exact.
 *
 * Layout (include/rpp/views/batch.hpp:49-68, dense_graded_vector_view.hpp):
 * tensor b of a batch lives at data + b*stride; coefficient index i is the
 * position in the full graded basis, degree-major and lexicographic within a
 * degree, so degree n starts at degree_begin[n] = (W^n - 1)/(W - 1).  A view
 * carries a degree range [min_degree, max_degree]: coefficients outside the
 * range read as zero and are never written.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAX_DEPTH 32

typedef struct {
    double* data;
    int64_t stride;
    int32_t min_degree;
    int32_t max_degree;
} orc_arg;

typedef struct {
    int32_t width;
    int32_t depth;
    int64_t db[ORC_MAX_DEPTH + 2]; /* degree_begin, depth+2 entries */
    int64_t pw[ORC_MAX_DEPTH + 2]; /* W^n */
} orc_basis;

/* include/rpp/basis/tensor_basis.hpp:122-130 (tensor_dimension) and
 * graded_basis.hpp:39-55 (start/end/size of degree). */
static void basis_init(orc_basis* b, int32_t width, int32_t depth) {
    b->width = width;
    b->depth = depth;
    b->db[0] = 0;
    b->pw[0] = 1;
    for (int n = 0; n <= depth; ++n) {
        b->db[n + 1] = b->db[n] + b->pw[n];
        b->pw[n + 1] = b->pw[n] * width;
    }
}

int64_t orc_tensor_dim(int32_t width, int32_t depth) {
    orc_basis b;
    basis_init(&b, width, depth);
    return b.db[depth + 1];
}

void orc_degree_begin(int32_t width, int32_t depth, int64_t* out) {
    orc_basis b;
    basis_init(&b, width, depth);
    for (int n = 0; n <= depth + 1; ++n) out[n] = b.db[n];
}

/* tensor_basis.hpp:93-102: digits of a level index read in reverse. */
int64_t orc_reverse_index(int32_t width, int32_t degree, int64_t idx) {
    int64_t r = 0;
    for (int d = 0; d < degree; ++d) {
        r = r * width + idx % width;
        idx /= width;
    }
    return r;
}

static int in_range(int32_t d, int32_t lo, int32_t hi) { return lo <= d && d <= hi; }

static int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }
static int32_t imin(int32_t a, int32_t b) { return a < b ? a : b; }

/* Word-split product at one output coefficient: sum over splits w = uv with
 * |u| in lhs's range and |v| in rhs's range of lhs[u]*rhs[v]
 * (cpu_typed_ft_ops_test_helper.hpp:160-205; gpu/block/operations/basic/
 * detail/ft_multiply.hpp:14-64 for the zero extension). */
static double split_sum(const orc_basis* B, const double* lhs, int32_t lmin, int32_t lmax,
                        const double* rhs, int32_t rmin, int32_t rmax, int32_t degree,
                        int64_t level_idx) {
    double acc = 0.0;
    for (int32_t ld = 0; ld <= degree; ++ld) {
        int32_t rd = degree - ld;
        if (!in_range(ld, lmin, lmax) || !in_range(rd, rmin, rmax)) continue;
        int64_t split = B->pw[rd];
        int64_t li = level_idx / split;
        int64_t ri = level_idx % split;
        acc += lhs[B->db[ld] + li] * rhs[B->db[rd] + ri];
    }
    return acc;
}

/* ---------------------------------------------------------------------------
 * Per-tensor operations.  Each works on one batch element.
 * ------------------------------------------------------------------------- */

/* out = alpha*a + beta*(b (x) c) on out's degree range; a may be NULL (ft_mul).
 * operations/basic/ft_fma.hpp:13-83, ft_mul.hpp:16-79 (ft_mul = fma with
 * alpha = 0), cpu/single_thread/operations/basic/ft_fma.hpp:22-65. */
static void one_fma(const orc_basis* B, double* out, int32_t omin, int32_t omax,
                    const double* a, int32_t amin, int32_t amax, const double* b, int32_t bmin,
                    int32_t bmax, const double* c, int32_t cmin, int32_t cmax, double alpha,
                    double beta) {
    for (int32_t n = omin; n <= omax && n <= B->depth; ++n) {
        for (int64_t i = 0; i < B->pw[n]; ++i) {
            double acc = 0.0;
            if (a && in_range(n, amin, amax)) acc = alpha * a[B->db[n] + i];
            acc += beta * split_sum(B, b, bmin, bmax, c, cmin, cmax, n, i);
            out[B->db[n] + i] = acc;
        }
    }
}

/* In-place product lhs <- beta * lhs (x) rhs on lhs's range, all reads of lhs
 * taken before any write (operations/basic/ft_inplace_mul.hpp:15-69; the
 * descending-degree order of gpu/block/operations/basic/ft_inplace_mul.hpp:
 * 46-58 guarantees exactly this). */
static void one_inplace_mul(const orc_basis* B, double* lhs, int32_t lmin, int32_t lmax,
                            const double* rhs, int32_t rmin, int32_t rmax, double beta,
                            double* scratch) {
    memcpy(scratch, lhs, sizeof(double) * (size_t)B->db[B->depth + 1]);
    for (int32_t n = lmin; n <= lmax && n <= B->depth; ++n)
        for (int64_t i = 0; i < B->pw[n]; ++i)
            lhs[B->db[n] + i] = beta * split_sum(B, scratch, lmin, lmax, rhs, rmin, rmax, n, i);
}

/* The three in-place FMA kinds of operations/basic/ft_inplace_fma.hpp:17-21:
 *   kind 0 (AEqualsBCPlusA): a <- alpha*a + beta*b(x)c
 *   kind 1 (AEqualsABPlusC): a <- alpha*c + beta*a(x)b
 *   kind 2 (AEqualsBAPlusC): a <- alpha*c + beta*b(x)a
 * Only a's range is written (gpu/block/operations/basic/ft_inplace_fma.hpp:
 * 48-131). */
static void one_inplace_fma(const orc_basis* B, int kind, double* a, int32_t amin, int32_t amax,
                            const double* b, int32_t bmin, int32_t bmax, const double* c,
                            int32_t cmin, int32_t cmax, double alpha, double beta,
                            double* scratch) {
    memcpy(scratch, a, sizeof(double) * (size_t)B->db[B->depth + 1]);
    for (int32_t n = amin; n <= amax && n <= B->depth; ++n) {
        for (int64_t i = 0; i < B->pw[n]; ++i) {
            double prod, add = 0.0;
            if (kind == 0) {
                prod = split_sum(B, b, bmin, bmax, c, cmin, cmax, n, i);
                add = alpha * scratch[B->db[n] + i];
            } else if (kind == 1) {
                prod = split_sum(B, scratch, amin, amax, b, bmin, bmax, n, i);
                if (in_range(n, cmin, cmax)) add = alpha * c[B->db[n] + i];
            } else {
                prod = split_sum(B, b, bmin, bmax, scratch, amin, amax, n, i);
                if (in_range(n, cmin, cmax)) add = alpha * c[B->db[n] + i];
            }
            a[B->db[n] + i] = add + beta * prod;
        }
    }
}

/* gpu/block/operations/linalg/vector_assign.hpp:51-112: copy the overlap of the
 * two ranges, zero the rest of out's range. */
static void one_assign(const orc_basis* B, double* out, int32_t omin, int32_t omax,
                       const double* arg, int32_t amin, int32_t amax) {
    for (int32_t n = omin; n <= omax && n <= B->depth; ++n)
        for (int64_t i = 0; i < B->pw[n]; ++i)
            out[B->db[n] + i] = in_range(n, amin, amax) ? arg[B->db[n] + i] : 0.0;
}

/* tensor_set_identity.hpp / tensor_add_identity.hpp: degree-0 slot only, and
 * only when the view holds degree 0. */
static void one_set_zero(const orc_basis* B, double* out, int32_t omin, int32_t omax) {
    for (int32_t n = omin; n <= omax && n <= B->depth; ++n)
        for (int64_t i = 0; i < B->pw[n]; ++i) out[B->db[n] + i] = 0.0;
}

/* operations/intermediate/ft_exp.hpp:66-81 (Horner: set_identity, then for
 * d = D..1: out <- out (x) arg[1..] / d, add_identity). */
static void one_exp(const orc_basis* B, double* out, int32_t omin, int32_t omax,
                    const double* arg, int32_t amin, int32_t amax, double* scratch) {
    const int32_t D = B->depth;
    one_set_zero(B, out, omin, omax);
    if (omin == 0) out[0] = 1.0;
    for (int32_t d = D; d > 0; --d) {
        one_inplace_mul(B, out, omin, omax, arg, imax(1, amin), imin(D, amax), 1.0 / d, scratch);
        if (omin == 0) out[0] += 1.0;
    }
}

/* operations/intermediate/ft_fmexp.hpp:66-87: out = multiplier (x) exp(X).
 * Assign, then for d = D..1: out <- multiplier + out (x) X[1..D-d+1] / d. */
static void one_fmexp(const orc_basis* B, double* out, int32_t omin, int32_t omax,
                      const double* mult, int32_t mmin, int32_t mmax, const double* x,
                      int32_t xmin, int32_t xmax, double* scratch) {
    const int32_t D = B->depth;
    one_assign(B, out, omin, omax, mult, mmin, mmax);
    for (int32_t d = D; d > 0; --d) {
        int32_t tmax = D - d + 1;
        one_inplace_fma(B, 1, out, omin, omax, x, imax(1, xmin), imin(tmax, xmax), mult, mmin,
                        mmax, 1.0, 1.0 / d, scratch);
    }
}

/* operations/intermediate/ft_log.hpp:87-114: set zero; for d = D..1:
 * add_identity((-1)^{d+1}/d); out[0..D-d+1] <- out (x) arg[1..D-d+1]. */
static void one_log(const orc_basis* B, double* out, int32_t omin, int32_t omax,
                    const double* arg, int32_t amin, int32_t amax, double* scratch) {
    const int32_t D = B->depth;
    one_set_zero(B, out, omin, omax);
    for (int32_t d = D; d > 0; --d) {
        int32_t tmax = D - d + 1;
        double val = ((d % 2 == 0) ? -1.0 : 1.0) / d;
        if (omin == 0) out[0] += val;
        one_inplace_mul(B, out, omin, imin(omax, tmax), arg, imax(1, amin), imin(tmax, amax), 1.0,
                        scratch);
    }
}

/* Adjoints of left/right multiplication (tests/rpp/ft_adjoint_test_helper.hpp:
 * 55-87; cpu/single_thread/operations/basic/ft_adj_lmul.hpp:40-115).
 *   left:  out[v] = sum_u op[u] arg[uv]
 *   right: out[u] = sum_v op[v] arg[uv]
 * out is zeroed on its range first. */
static void one_adjoint(const orc_basis* B, int left, double* out, int32_t omin, int32_t omax,
                        const double* op, int32_t pmin, int32_t pmax, const double* arg,
                        int32_t amin, int32_t amax) {
    one_set_zero(B, out, omin, omax);
    for (int32_t ad = amin; ad <= amax && ad <= B->depth; ++ad) {
        for (int32_t pd = pmin; pd <= pmax && pd <= ad; ++pd) {
            int32_t od = ad - pd;
            if (!in_range(od, omin, omax)) continue;
            int64_t suffix = B->pw[left ? od : pd];
            for (int64_t i = 0; i < B->pw[ad]; ++i) {
                int64_t pre = i / suffix, suf = i % suffix;
                int64_t pi = left ? pre : suf, oi = left ? suf : pre;
                out[B->db[od] + oi] += op[B->db[pd] + pi] * arg[B->db[ad] + i];
            }
        }
    }
}

/* operations/basic/tensor_generalised_antipode.hpp:14-81 and cpu/single_thread/
 * operations/basic/tensor_generalised_antipode.hpp:44-72:
 * out[rev w] = (-1)^{|w|} arg[w] (signed) or arg[w] (reflect) on out's range;
 * degrees missing from arg are zeroed. */
static void one_antipode(const orc_basis* B, int signed_, double* out, int32_t omin, int32_t omax,
                         const double* arg, int32_t amin, int32_t amax) {
    for (int32_t n = omin; n <= omax && n <= B->depth; ++n) {
        if (!in_range(n, amin, amax)) {
            for (int64_t i = 0; i < B->pw[n]; ++i) out[B->db[n] + i] = 0.0;
            continue;
        }
        double sign = (signed_ && (n % 2)) ? -1.0 : 1.0;
        for (int64_t i = 0; i < B->pw[n]; ++i)
            out[B->db[n] + orc_reverse_index(B->width, n, i)] = sign * arg[B->db[n] + i];
    }
}

/* ---------------------------------------------------------------------------
 * Batched entry points (ctypes).  Scratch is per call.
 * ------------------------------------------------------------------------- */

#define ORC_PTR(arg, b) ((arg)->data + (int64_t)(b) * (arg)->stride)

int orc_ft_fma(int32_t W, int32_t D, int64_t batch, const orc_arg* out, const orc_arg* a,
               const orc_arg* b, const orc_arg* c, double alpha, double beta) {
    orc_basis B;
    basis_init(&B, W, D);
    for (int64_t k = 0; k < batch; ++k)
        one_fma(&B, ORC_PTR(out, k), out->min_degree, out->max_degree, a ? ORC_PTR(a, k) : NULL,
                a ? a->min_degree : 0, a ? a->max_degree : -1, ORC_PTR(b, k), b->min_degree,
                b->max_degree, ORC_PTR(c, k), c->min_degree, c->max_degree, alpha, beta);
    return 0;
}

int orc_ft_inplace_fma(int32_t W, int32_t D, int64_t batch, int kind, const orc_arg* a,
                       const orc_arg* b, const orc_arg* c, double alpha, double beta) {
    orc_basis B;
    basis_init(&B, W, D);
    double* s = (double*)malloc(sizeof(double) * (size_t)B.db[D + 1]);
    for (int64_t k = 0; k < batch; ++k)
        one_inplace_fma(&B, kind, ORC_PTR(a, k), a->min_degree, a->max_degree, ORC_PTR(b, k),
                        b->min_degree, b->max_degree, ORC_PTR(c, k), c->min_degree, c->max_degree,
                        alpha, beta, s);
    free(s);
    return 0;
}

int orc_ft_inplace_mul(int32_t W, int32_t D, int64_t batch, const orc_arg* lhs, const orc_arg* rhs,
                       double beta) {
    orc_basis B;
    basis_init(&B, W, D);
    double* s = (double*)malloc(sizeof(double) * (size_t)B.db[D + 1]);
    for (int64_t k = 0; k < batch; ++k)
        one_inplace_mul(&B, ORC_PTR(lhs, k), lhs->min_degree, lhs->max_degree, ORC_PTR(rhs, k),
                        rhs->min_degree, rhs->max_degree, beta, s);
    free(s);
    return 0;
}

int orc_ft_exp(int32_t W, int32_t D, int64_t batch, const orc_arg* out, const orc_arg* arg) {
    orc_basis B;
    basis_init(&B, W, D);
    double* s = (double*)malloc(sizeof(double) * (size_t)B.db[D + 1]);
    for (int64_t k = 0; k < batch; ++k)
        one_exp(&B, ORC_PTR(out, k), out->min_degree, out->max_degree, ORC_PTR(arg, k),
                arg->min_degree, arg->max_degree, s);
    free(s);
    return 0;
}

int orc_ft_fmexp(int32_t W, int32_t D, int64_t batch, const orc_arg* out, const orc_arg* mult,
                 const orc_arg* x) {
    orc_basis B;
    basis_init(&B, W, D);
    double* s = (double*)malloc(sizeof(double) * (size_t)B.db[D + 1]);
    for (int64_t k = 0; k < batch; ++k)
        one_fmexp(&B, ORC_PTR(out, k), out->min_degree, out->max_degree, ORC_PTR(mult, k),
                  mult->min_degree, mult->max_degree, ORC_PTR(x, k), x->min_degree, x->max_degree,
                  s);
    free(s);
    return 0;
}

int orc_ft_log(int32_t W, int32_t D, int64_t batch, const orc_arg* out, const orc_arg* arg) {
    orc_basis B;
    basis_init(&B, W, D);
    double* s = (double*)malloc(sizeof(double) * (size_t)B.db[D + 1]);
    for (int64_t k = 0; k < batch; ++k)
        one_log(&B, ORC_PTR(out, k), out->min_degree, out->max_degree, ORC_PTR(arg, k),
                arg->min_degree, arg->max_degree, s);
    free(s);
    return 0;
}

int orc_ft_adjoint(int32_t W, int32_t D, int64_t batch, int left, const orc_arg* out,
                   const orc_arg* op, const orc_arg* arg) {
    orc_basis B;
    basis_init(&B, W, D);
    for (int64_t k = 0; k < batch; ++k)
        one_adjoint(&B, left, ORC_PTR(out, k), out->min_degree, out->max_degree, ORC_PTR(op, k),
                    op->min_degree, op->max_degree, ORC_PTR(arg, k), arg->min_degree,
                    arg->max_degree);
    return 0;
}

int orc_antipode(int32_t W, int32_t D, int64_t batch, int signed_, const orc_arg* out,
                 const orc_arg* arg) {
    orc_basis B;
    basis_init(&B, W, D);
    for (int64_t k = 0; k < batch; ++k)
        one_antipode(&B, signed_, ORC_PTR(out, k), out->min_degree, out->max_degree,
                     ORC_PTR(arg, k), arg->min_degree, arg->max_degree);
    return 0;
}

/* Sparse matrix-vector products with the CPU strategy's begin-relative
 * indexing: out.begin()[row], arg.begin()[col]
 * (cpu/single_thread/operations/linalg/sparse_matrix_vector.hpp:57-86 for CSR,
 * :138-163 for CSC).  out_begin/arg_begin are the view begin offsets
 * (degree_begin of the views' minimum degrees); out_len is the view size, which
 * the CSC form zeroes first. */
int orc_spmv(int64_t batch, int csc, int64_t outer_dim, const int64_t* offsets,
             const int64_t* indices, const double* values, double* out, int64_t out_stride,
             int64_t out_begin, int64_t out_len, const double* arg, int64_t arg_stride,
             int64_t arg_begin, double alpha) {
    for (int64_t k = 0; k < batch; ++k) {
        double* o = out + k * out_stride + out_begin;
        const double* x = arg + k * arg_stride + arg_begin;
        if (!csc) {
            for (int64_t r = 0; r < outer_dim; ++r) {
                double acc = 0.0;
                for (int64_t e = offsets[r]; e < offsets[r + 1]; ++e) acc += values[e] * x[indices[e]];
                o[r] = alpha * acc;
            }
        } else {
            for (int64_t i = 0; i < out_len; ++i) o[i] = 0.0;
            for (int64_t col = 0; col < outer_dim; ++col) {
                double xv = alpha * x[col];
                for (int64_t e = offsets[col]; e < offsets[col + 1]; ++e) o[indices[e]] += values[e] * xv;
            }
        }
    }
    return 0;
}

/* ---------------------------------------------------------------------------
 * Signatures of piecewise-linear paths (the Chen loop a caller writes over
 * ft_fmexp: tests/rpp/gpu/block/ops/ft_fmexp_tests.cu:126-147), and the
 * stored-prefix reverse pass composed from ft_adj_lmul / ft_adj_rmul and the
 * derivative of the letter-only exponential.
 * ------------------------------------------------------------------------- */

/* exp of a letter-only tensor: E[w] = prod_i x[w_i] / |w|!  (the closed form
 * of ft_exp.hpp:66-81 for an argument that lives in degree one). */
static void letter_exp(const orc_basis* B, const double* x, double* E) {
    E[0] = 1.0;
    for (int32_t n = 1; n <= B->depth; ++n) {
        double inv = 1.0 / n;
        for (int64_t i = 0; i < B->pw[n]; ++i)
            E[B->db[n] + i] = E[B->db[n - 1] + i / B->width] * x[i % B->width] * inv;
    }
}

/* S <- S (x) exp(x) for a letter-only increment, in place, by the per-level
 * Horner chains (level n: T_0 = S_0, T_j = S_j + T_{j-1} (x) x/(n-j+1),
 * new S_n = T_n), levels written from the top down. */
static void chen_step(const orc_basis* B, double* S, const double* x, double* T0, double* T1) {
    const int32_t D = B->depth, W = B->width;
    for (int32_t n = D; n >= 1; --n) {
        double* prev = T0;
        double* cur = T1;
        prev[0] = S[0];
        for (int32_t j = 1; j <= n; ++j) {
            double c = 1.0 / (n - j + 1);
            for (int64_t i = 0; i < B->pw[j]; ++i)
                cur[i] = S[B->db[j] + i] + prev[i / W] * (x[i % W] * c);
            double* t = prev;
            prev = cur;
            cur = t;
        }
        memcpy(S + B->db[n], prev, sizeof(double) * (size_t)B->pw[n]);
    }
}

/* Forward signature of one path from the unit tensor. */
static void one_signature(const orc_basis* B, const double* incr, int64_t len, double* S,
                          double* T0, double* T1) {
    memset(S, 0, sizeof(double) * (size_t)B->db[B->depth + 1]);
    S[0] = 1.0;
    for (int64_t k = 0; k < len; ++k) chen_step(B, S, incr + k * B->width, T0, T1);
}

/* Reverse pass for loss = <ell, S(x)> with stored prefixes:
 *   G_L = ell;  for k = L..1:
 *     H = adj_lmul(S_{k-1}, G_k)            (d loss / d E_k)
 *     grad x_k = H contracted with d E_k / d x_k
 *     G_{k-1} = adj_rmul(E_k, G_k). */
static void one_signature_grad(const orc_basis* B, const double* incr, int64_t len,
                               const double* ell, double* grad, double* work) {
    const int64_t dim = B->db[B->depth + 1];
    const int32_t W = B->width, D = B->depth;
    double* prefixes = (double*)malloc(sizeof(double) * (size_t)(dim * (len + 1)));
    double* G = work;
    double* Gn = work + dim;
    double* H = work + 2 * dim;
    double* E = work + 3 * dim;
    double* T0 = work + 4 * dim;
    double* T1 = work + 5 * dim;
    memset(prefixes, 0, sizeof(double) * (size_t)dim);
    prefixes[0] = 1.0;
    for (int64_t k = 0; k < len; ++k) {
        memcpy(prefixes + (k + 1) * dim, prefixes + k * dim, sizeof(double) * (size_t)dim);
        chen_step(B, prefixes + (k + 1) * dim, incr + k * W, T0, T1);
    }
    memcpy(G, ell, sizeof(double) * (size_t)dim);
    for (int64_t k = len - 1; k >= 0; --k) {
        const double* x = incr + k * W;
        letter_exp(B, x, E);
        one_adjoint(B, 1, H, 0, D, prefixes + k * dim, 0, D, G, 0, D);
        /* dE[w]/dx_a = sum over positions p with w_p = a of prod_{i != p} x[w_i] / |w|! */
        double* g = grad + k * W;
        for (int32_t a = 0; a < W; ++a) g[a] = 0.0;
        for (int32_t n = 1; n <= D; ++n) {
            double fact = 1.0;
            for (int32_t m = 2; m <= n; ++m) fact *= m;
            for (int64_t i = 0; i < B->pw[n]; ++i) {
                double h = H[B->db[n] + i];
                if (h == 0.0) continue;
                int letters[ORC_MAX_DEPTH];
                double before[ORC_MAX_DEPTH + 1], after[ORC_MAX_DEPTH + 1];
                int64_t t = i;
                for (int32_t p = n - 1; p >= 0; --p) {
                    letters[p] = (int)(t % W);
                    t /= W;
                }
                /* prod_{q != p} x[w_q] = (prod_{q < p}) * (prod_{q > p}) */
                before[0] = 1.0;
                for (int32_t p = 0; p < n; ++p) before[p + 1] = before[p] * x[letters[p]];
                after[n] = 1.0;
                for (int32_t p = n - 1; p >= 0; --p) after[p] = after[p + 1] * x[letters[p]];
                double hs = h / fact;
                for (int32_t p = 0; p < n; ++p) g[letters[p]] += hs * before[p] * after[p + 1];
            }
        }
        one_adjoint(B, 0, Gn, 0, D, E, 0, D, G, 0, D);
        double* tmp = G;
        G = Gn;
        Gn = tmp;
    }
    free(prefixes);
}

typedef struct {
    const orc_basis* B;
    const double* incr;
    const int64_t* offsets;
    const double* ell;
    double* sig;
    double* grad;
    int64_t begin, end;
    int want_grad;
} orc_sig_job;

static void* sig_worker(void* p) {
    orc_sig_job* j = (orc_sig_job*)p;
    const int64_t dim = j->B->db[j->B->depth + 1];
    const int32_t W = j->B->width;
    double* work = (double*)malloc(sizeof(double) * (size_t)(6 * dim));
    for (int64_t b = j->begin; b < j->end; ++b) {
        int64_t off = j->offsets[b], len = j->offsets[b + 1] - off;
        if (j->sig)
            one_signature(j->B, j->incr + off * W, len, j->sig + b * dim, work, work + dim);
        if (j->want_grad)
            one_signature_grad(j->B, j->incr + off * W, len, j->ell + b * dim, j->grad + off * W,
                               work);
    }
    free(work);
    return NULL;
}

/* Batched signatures over a ragged batch: path b has increments
 * incr[offsets[b]*W .. offsets[b+1]*W).  sig (B x dim, may be NULL) receives
 * S(x_b); when ell (B x dim) and grad (offsets[B] x W) are given, grad receives
 * d/dx of sum_b <ell_b, S(x_b)>.  threads > 1 splits the batch over pthreads. */
int orc_signature(int32_t W, int32_t D, int64_t batch, const double* incr, const int64_t* offsets,
                  double* sig, const double* ell, double* grad, int32_t threads) {
    orc_basis B;
    basis_init(&B, W, D);
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    orc_sig_job jobs[256];
    int64_t per = (batch + threads - 1) / threads;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        orc_sig_job* j = &jobs[t];
        j->B = &B;
        j->incr = incr;
        j->offsets = offsets;
        j->ell = ell;
        j->sig = sig;
        j->grad = grad;
        j->want_grad = (ell != NULL && grad != NULL);
        j->begin = t * per;
        j->end = (t + 1) * per < batch ? (t + 1) * per : batch;
        if (j->begin >= j->end) break;
        if (threads == 1) {
            sig_worker(j);
        } else {
            pthread_create(&tid[t], NULL, sig_worker, j);
            ++started;
        }
    }
    for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Shuffle algebra.  Each coefficient is enumerated over subsets of letter
 * positions, first letter first, the way the reference's own test references
 * do (tests/rpp/shuffle_adjoint_test_helper.hpp:49-94 and
 * tests/rpp/half_shuffle_adjoint_test_helper.hpp:12-80), independently of
 * the operation's masked index packing.
 * ------------------------------------------------------------------------- */

/* Letters of a level index, first letter first. */
static void word_letters(const orc_basis* B, int32_t n, int64_t idx, int32_t* w) {
    for (int32_t p = n - 1; p >= 0; --p) {
        w[p] = (int32_t)(idx % B->width);
        idx /= B->width;
    }
}

/* Split the word w (n letters) by the position subset `mask` (bit p = letter
 * p, first letter = bit 0): the letters in the subset form `sel`, the others
 * `rest`, both in order.  Returns |sel|. */
static int32_t split_word(const orc_basis* B, const int32_t* w, int32_t n, uint64_t mask,
                          int64_t* sel, int64_t* rest) {
    int32_t k = 0;
    *sel = 0;
    *rest = 0;
    for (int32_t p = 0; p < n; ++p) {
        if ((mask >> p) & 1u) {
            *sel = *sel * B->width + w[p];
            ++k;
        } else {
            *rest = *rest * B->width + w[p];
        }
    }
    return k;
}

/* (lhs sh rhs)[w] = sum over position subsets S of lhs[w|S] rhs[w|S^c], terms
 * whose degrees fall outside an operand's range omitted
 * (operations/implementation/word_shuffle_product.hpp:43-97).  With
 * `half`, position 0 always goes to lhs: the left half-shuffle coefficient
 * (operations/implementation/word_half_shuffle_product.hpp:12-56). */
static double shuffle_coeff(const orc_basis* B, int32_t n, int64_t idx, const double* lhs,
                            int32_t lmin, int32_t lmax, const double* rhs, int32_t rmin,
                            int32_t rmax, int half) {
    int32_t w[ORC_MAX_DEPTH];
    word_letters(B, n, idx, w);
    double acc = 0.0;
    for (uint64_t mask = 0; mask < ((uint64_t)1 << n); ++mask) {
        if (half && !(mask & 1u)) continue;
        int64_t li, ri;
        int32_t kl = split_word(B, w, n, mask, &li, &ri);
        int32_t kr = n - kl;
        if (!in_range(kl, lmin, lmax) || !in_range(kr, rmin, rmax)) continue;
        acc += lhs[B->db[kl] + li] * rhs[B->db[kr] + ri];
    }
    return acc;
}

/* cpu/single_thread/operations/basic/st_mul.hpp:44-69 (mode 0: out = beta
 * lhs sh rhs), st_fma.hpp:44-80 (mode 1: out = alpha a + beta b sh c) and
 * st_inplace_fma.hpp:44-70 (mode 2: a = alpha a + beta b sh c, `out` is a). */
static void one_st(const orc_basis* B, int mode, double* out, int32_t omin, int32_t omax,
                   const double* a, int32_t amin, int32_t amax, const double* b, int32_t bmin,
                   int32_t bmax, const double* c, int32_t cmin, int32_t cmax, double alpha,
                   double beta) {
    for (int32_t n = omin; n <= omax && n <= B->depth; ++n) {
        for (int64_t i = 0; i < B->pw[n]; ++i) {
            double prod = shuffle_coeff(B, n, i, b, bmin, bmax, c, cmin, cmax, 0);
            double v = beta * prod;
            if (mode == 1 && a && in_range(n, amin, amax)) v += alpha * a[B->db[n] + i];
            if (mode == 2) v += alpha * out[B->db[n] + i];
            out[B->db[n] + i] = v;
        }
    }
}

/* cpu/single_thread/operations/basic/left_hs_mul.hpp:44-84: out[0] = 0 and
 * out[a v] = beta (integrator < integrand)[a v]. */
static void one_left_hs_mul(const orc_basis* B, double* out, int32_t omin, int32_t omax,
                            const double* x, int32_t xmin, int32_t xmax, const double* y,
                            int32_t ymin, int32_t ymax, double beta) {
    for (int32_t n = omin; n <= omax && n <= B->depth; ++n) {
        for (int64_t i = 0; i < B->pw[n]; ++i)
            out[B->db[n] + i] = n == 0 ? 0.0 : beta * shuffle_coeff(B, n, i, x, xmin, xmax, y, ymin, ymax, 1);
    }
}

/* cpu/single_thread/operations/basic/st_adj_mul.hpp:46-85 with
 * operations/implementation/shuffle_adjoint_op_loop.hpp and
 * word_shuffle_adjoint_multiply.hpp: out[w] = sum_u op[u] sum_{s in w sh u}
 * arg[s], i.e. <out, x> = <arg, op sh x>.  Written as the transpose of the
 * shuffle product: every arg word s and position subset S send
 * op[s|S] arg[s] to out[s|S^c]. */
static void one_st_adj_mul(const orc_basis* B, double* out, int32_t omin, int32_t omax,
                           const double* op, int32_t pmin, int32_t pmax, const double* arg,
                           int32_t amin, int32_t amax) {
    one_set_zero(B, out, omin, omax);
    int32_t w[ORC_MAX_DEPTH];
    for (int32_t N = amin; N <= amax && N <= B->depth; ++N) {
        for (int64_t s = 0; s < B->pw[N]; ++s) {
            word_letters(B, N, s, w);
            for (uint64_t mask = 0; mask < ((uint64_t)1 << N); ++mask) {
                int64_t pi, oi;
                int32_t kp = split_word(B, w, N, mask, &pi, &oi);
                int32_t ko = N - kp;
                if (!in_range(kp, pmin, pmax) || !in_range(ko, omin, omax)) continue;
                out[B->db[ko] + oi] += op[B->db[kp] + pi] * arg[B->db[N] + s];
            }
        }
    }
}

/* The adjoints of the left half-shuffle x < y with respect to each factor,
 * as the transpose of the forward product: every arg word s (degree >= 1)
 * and split of its positions 1.. into (left rest, right) with position 0
 * on the left.
 *   fixed_left  (cpu/single_thread/operations/basic/left_hs_adj_lmul.hpp:
 *               73-124): out = y-cotangent, out[right] += beta x[left] arg[s]
 *               with x = `fixed` (the integrator) and arg = the integrand
 *               cotangent;
 *   !fixed_left (left_hs_adj_rmul.hpp:44-106): out = x-cotangent,
 *               out[left] += beta y[right] arg[s] with y = `fixed` (the
 *               integrand) and arg = the integrator cotangent; out[0] = 0. */
static void one_left_hs_adjoint(const orc_basis* B, int fixed_left, double* out, int32_t omin,
                                int32_t omax, const double* fixed, int32_t fmin, int32_t fmax,
                                const double* arg, int32_t amin, int32_t amax, double beta) {
    one_set_zero(B, out, omin, omax);
    int32_t w[ORC_MAX_DEPTH];
    for (int32_t N = imax(amin, 1); N <= amax && N <= B->depth; ++N) {
        for (int64_t s = 0; s < B->pw[N]; ++s) {
            word_letters(B, N, s, w);
            for (uint64_t mask = 1; mask < ((uint64_t)1 << N); mask += 2) {
                int64_t li, ri;
                int32_t kl = split_word(B, w, N, mask, &li, &ri);
                int32_t kr = N - kl;
                int32_t kf = fixed_left ? kl : kr, ko = fixed_left ? kr : kl;
                int64_t fi = fixed_left ? li : ri, oi = fixed_left ? ri : li;
                if (!in_range(kf, fmin, fmax) || !in_range(ko, omin, omax)) continue;
                out[B->db[ko] + oi] += beta * fixed[B->db[kf] + fi] * arg[B->db[N] + s];
            }
        }
    }
}

int orc_st(int32_t W, int32_t D, int64_t batch, int mode, const orc_arg* out, const orc_arg* a,
           const orc_arg* b, const orc_arg* c, double alpha, double beta) {
    orc_basis B;
    basis_init(&B, W, D);
    for (int64_t k = 0; k < batch; ++k)
        one_st(&B, mode, ORC_PTR(out, k), out->min_degree, out->max_degree, a ? ORC_PTR(a, k) : NULL,
               a ? a->min_degree : 1, a ? a->max_degree : 0, ORC_PTR(b, k), b->min_degree,
               b->max_degree, ORC_PTR(c, k), c->min_degree, c->max_degree, alpha, beta);
    return 0;
}

int orc_left_hs_mul(int32_t W, int32_t D, int64_t batch, const orc_arg* out, const orc_arg* x,
                    const orc_arg* y, double beta) {
    orc_basis B;
    basis_init(&B, W, D);
    for (int64_t k = 0; k < batch; ++k)
        one_left_hs_mul(&B, ORC_PTR(out, k), out->min_degree, out->max_degree, ORC_PTR(x, k),
                        x->min_degree, x->max_degree, ORC_PTR(y, k), y->min_degree, y->max_degree,
                        beta);
    return 0;
}

int orc_st_adj_mul(int32_t W, int32_t D, int64_t batch, const orc_arg* out, const orc_arg* op,
                   const orc_arg* arg) {
    orc_basis B;
    basis_init(&B, W, D);
    for (int64_t k = 0; k < batch; ++k)
        one_st_adj_mul(&B, ORC_PTR(out, k), out->min_degree, out->max_degree, ORC_PTR(op, k),
                       op->min_degree, op->max_degree, ORC_PTR(arg, k), arg->min_degree,
                       arg->max_degree);
    return 0;
}

/* lmul: (out, integrator, integrand) = (out, fixed x, cotangent);
 * rmul: (out, integrator, integrand) = (out, cotangent, fixed y) -- the
 * argument order of the reference's operator() in both cases. */
int orc_left_hs_adjoint(int32_t W, int32_t D, int64_t batch, int lmul, const orc_arg* out,
                        const orc_arg* integrator, const orc_arg* integrand, double beta) {
    orc_basis B;
    basis_init(&B, W, D);
    const orc_arg* fixed = lmul ? integrator : integrand;
    const orc_arg* cot = lmul ? integrand : integrator;
    for (int64_t k = 0; k < batch; ++k)
        one_left_hs_adjoint(&B, lmul, ORC_PTR(out, k), out->min_degree, out->max_degree,
                            ORC_PTR(fixed, k), fixed->min_degree, fixed->max_degree, ORC_PTR(cot, k),
                            cot->min_degree, cot->max_degree, beta);
    return 0;
}

/* cpu/single_thread/operations/basic/tensor_pairing.hpp:40-72: result[b] =
 * sum of functional[i] arg[i] over the degrees both views hold. */
int orc_tensor_pairing(int32_t W, int32_t D, int64_t batch, double* result, const orc_arg* f,
                       const orc_arg* a) {
    orc_basis B;
    basis_init(&B, W, D);
    int32_t lo = imax(f->min_degree, a->min_degree);
    int32_t hi = imin(imin(f->max_degree, a->max_degree), D);
    for (int64_t k = 0; k < batch; ++k) {
        const double* fp = ORC_PTR(f, k);
        const double* ap = ORC_PTR(a, k);
        double acc = 0.0;
        if (lo <= hi)
            for (int64_t i = B.db[lo]; i < B.db[hi + 1]; ++i) acc += fp[i] * ap[i];
        result[k] = acc;
    }
    return 0;
}
