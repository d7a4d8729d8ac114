// ref_bridge.cpp -- extern "C" shim over the UNMODIFIED reference CPU strategy.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the
// reference's own headers (include/rpp/**) into oracle/_ref/librpp_ref.so; it
// is used only to pin the C oracle (rpp_oracle.c) and to generate the golden
// fixtures under tests/golden/.  Every function drives the reference's public
// operation API (rpp::ops::<op>(strategy, config, batches..., basis, n, ...))
// with rpp::cpu::strategies::SingleThreadStrategy<double>, exactly as a user
// of the reference would.  No reference source is copied here.
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include <rpp/basis/hall_basis.hpp>
#include <rpp/basis/lie_multiplication.hpp>
#include <rpp/basis/tensor_basis.hpp>
#include <rpp/cpu/single_thread/operations.hpp>
#include <rpp/cpu/strategies.hpp>
#include <rpp/operations.hpp>
#include <rpp/sparse/l2t_matrix.hpp>
#include <rpp/sparse/t2l_matrix.hpp>
#include <rpp/views/views.hpp>

namespace {

using Strategy = rpp::cpu::strategies::SingleThreadStrategy<double>;
using Arch = rpp::arch::NativeArchitecture;
using Index = Arch::Index;
using Degree = Arch::Degree;
using Basis = rpp::basis::TensorBasis<Arch>;

struct Arg {
    double* data;
    int64_t stride;
    int32_t min_degree;
    int32_t max_degree;
};

struct BasisData {
    std::vector<Index> degree_begin;
    Basis basis;
    BasisData(Degree w, Degree d) : degree_begin(make(w, d)), basis(w, d, degree_begin.data()) {}
    static std::vector<Index> make(Degree w, Degree d) {
        std::vector<Index> db(static_cast<size_t>(d) + 2);
        db[0] = 0;
        Index p = 1;
        for (Degree n = 0; n <= d; ++n) {
            db[n + 1] = db[n] + p;
            p *= w;
        }
        return db;
    }
};

auto batch(Arg const* a) {
    return rpp::make_tensor_batch(a->data, static_cast<Index>(a->stride), Degree{a->min_degree},
                                  Degree{a->max_degree});
}
auto cbatch(Arg const* a) {
    return rpp::make_tensor_batch(static_cast<double const*>(a->data), static_cast<Index>(a->stride),
                                  Degree{a->min_degree}, Degree{a->max_degree});
}

template <typename E>
int status(E const& err) {
    return err ? 0 : 1 + static_cast<int>(err.code());
}

}  // namespace

extern "C" {

int ref_ft_mul(int32_t W, int32_t D, int64_t n, Arg const* out, Arg const* lhs, Arg const* rhs,
               double beta) {
    BasisData bd(W, D);
    return status(
        rpp::ops::ft_mul(Strategy{}, {}, batch(out), cbatch(lhs), cbatch(rhs), bd.basis, n, beta));
}

int ref_ft_fma(int32_t W, int32_t D, int64_t n, Arg const* out, Arg const* a, Arg const* b,
               Arg const* c, double alpha, double beta) {
    BasisData bd(W, D);
    return status(rpp::ops::ft_fma(Strategy{}, {}, batch(out), cbatch(a), cbatch(b), cbatch(c),
                                   bd.basis, n, alpha, beta));
}

int ref_ft_inplace_fma(int32_t W, int32_t D, int64_t n, int kind, Arg const* a, Arg const* b,
                       Arg const* c, double alpha, double beta) {
    using T = rpp::ops::FTInplaceFMAType;
    BasisData bd(W, D);
    if (kind == 0)
        return status(rpp::ops::ft_inplace_fma<T::AEqualsBCPlusA>(
            Strategy{}, {}, batch(a), cbatch(b), cbatch(c), bd.basis, n, alpha, beta));
    if (kind == 1)
        return status(rpp::ops::ft_inplace_fma<T::AEqualsABPlusC>(
            Strategy{}, {}, batch(a), cbatch(b), cbatch(c), bd.basis, n, alpha, beta));
    return status(rpp::ops::ft_inplace_fma<T::AEqualsBAPlusC>(
        Strategy{}, {}, batch(a), cbatch(b), cbatch(c), bd.basis, n, alpha, beta));
}

int ref_ft_inplace_mul(int32_t W, int32_t D, int64_t n, Arg const* lhs, Arg const* rhs,
                       double beta) {
    BasisData bd(W, D);
    return status(
        rpp::ops::ft_inplace_mul(Strategy{}, {}, batch(lhs), cbatch(rhs), bd.basis, n, beta));
}

int ref_ft_exp(int32_t W, int32_t D, int64_t n, Arg const* out, Arg const* arg) {
    BasisData bd(W, D);
    return status(rpp::ops::ft_exp(Strategy{}, {}, batch(out), cbatch(arg), bd.basis, n));
}

int ref_ft_fmexp(int32_t W, int32_t D, int64_t n, Arg const* out, Arg const* mult, Arg const* x) {
    BasisData bd(W, D);
    return status(
        rpp::ops::ft_fmexp(Strategy{}, {}, batch(out), cbatch(mult), cbatch(x), bd.basis, n));
}

int ref_ft_log(int32_t W, int32_t D, int64_t n, Arg const* out, Arg const* arg) {
    BasisData bd(W, D);
    return status(rpp::ops::ft_log(Strategy{}, {}, batch(out), cbatch(arg), bd.basis, n));
}

int ref_ft_adjoint(int32_t W, int32_t D, int64_t n, int left, Arg const* out, Arg const* op,
                   Arg const* arg) {
    BasisData bd(W, D);
    if (left)
        return status(
            rpp::ops::ft_adj_lmul(Strategy{}, {}, batch(out), cbatch(op), cbatch(arg), bd.basis, n));
    return status(
        rpp::ops::ft_adj_rmul(Strategy{}, {}, batch(out), cbatch(op), cbatch(arg), bd.basis, n));
}

int ref_antipode(int32_t W, int32_t D, int64_t n, int signed_, Arg const* out, Arg const* arg) {
    BasisData bd(W, D);
    if (signed_)
        return status(rpp::ops::tensor_antipode(Strategy{}, {}, batch(out), cbatch(arg), bd.basis, n));
    return status(rpp::ops::tensor_reflect(Strategy{}, {}, batch(out), cbatch(arg), bd.basis, n));
}

int64_t ref_reverse_index(int32_t W, int32_t D, int32_t degree, int64_t idx) {
    BasisData bd(W, D);
    return bd.basis.reverse_index(idx, degree);
}

// Hall basis tables: degree_begin (depth+2 entries) and the (left, right)
// parent pairs (2*true_size entries).  Returns true_size, or -1 if cap is short.
int64_t ref_hall_basis(int32_t W, int32_t D, int64_t* degree_begin, int64_t* pairs, int64_t cap) {
    rpp::basis::HallBasis<Arch> hall(W, D);
    auto lie = hall.to_lie_basis();
    const Index ts = lie.true_size();
    if (2 * ts > cap) return -1;
    for (Degree d = 0; d <= D + 1; ++d) degree_begin[d] = lie.degree_begin[d];
    for (Index k = 0; k < ts; ++k) {
        auto [l, r] = lie[k];
        pairs[2 * k] = l;
        pairs[2 * k + 1] = r;
    }
    return ts;
}

int64_t ref_find_bracket(int32_t W, int32_t D, int64_t left, int64_t right, int32_t hint) {
    rpp::basis::HallBasis<Arch> hall(W, D);
    return hall.to_lie_basis().find_bracket(left, right, hint);
}

// Sparse conversion matrices as built by the reference (CSC).  which = 0:
// make_t2l_matrix (rows = Lie idx, cols = tensor index); which = 1:
// make_l2t_matrix (rows = tensor index, cols = Lie idx).  Returns nnz, or -1
// if a capacity is short.  dims receives {nnz, outer_dim, inner_dim}.
int64_t ref_conversion_matrix(int32_t W, int32_t D, int which, int64_t* offsets, int64_t off_cap,
                              int64_t* indices, double* values, int64_t nnz_cap, int64_t* dims) {
    rpp::basis::HallBasis<Arch> hall(W, D);
    auto lie = hall.to_lie_basis();
    auto emit = [&](auto const& m) -> int64_t {
        const int64_t nnz = m.nnz(), outer = m.outer_dim();
        dims[0] = nnz;
        dims[1] = outer;
        dims[2] = m.inner_dim();
        if (nnz > nnz_cap || outer + 1 > off_cap) return -1;
        for (int64_t i = 0; i <= outer; ++i) offsets[i] = m.offsets()[i];
        for (int64_t i = 0; i < nnz; ++i) {
            indices[i] = m.indices()[i];
            values[i] = m.data()[i];
        }
        return nnz;
    };
    if (which == 0) {
        rpp::basis::LieMultiplicationCache<Arch> cache(lie);
        return emit(rpp::sparse::make_t2l_matrix<double>(lie, cache));
    }
    return emit(rpp::sparse::make_l2t_matrix<double>(lie));
}

// tensor_to_lie / lie_to_tensor through the reference front ends with a CSC
// GradedMatrixView over caller arrays.  Tensor views cover degrees
// [0, D]; Lie views cover [1, D] (slot 0 unused, begin-relative indexing).
int ref_tensor_lie(int32_t W, int32_t D, int64_t n, int to_lie, int64_t nnz, int64_t outer,
                   int64_t inner, int64_t const* offsets, int64_t const* indices,
                   double const* values, double* out, int64_t out_stride, double const* arg,
                   int64_t arg_stride) {
    BasisData bd(W, D);
    rpp::basis::HallBasis<Arch> hall(W, D);
    auto lie = hall.to_lie_basis();
    using M = rpp::sparse::GradedMatrixView<rpp::sparse::MatrixFormat::CSC, double const*,
                                            Index const*, Index const*>;
    M m(values, reinterpret_cast<Index const*>(indices), reinterpret_cast<Index const*>(offsets),
        static_cast<Index>(nnz), static_cast<Index>(outer), static_cast<Index>(inner));
    if (to_lie) {
        auto ob = rpp::make_lie_batch(out, static_cast<Index>(out_stride), Degree{1}, Degree{D});
        auto ab = rpp::make_tensor_batch(arg, static_cast<Index>(arg_stride), Degree{0}, Degree{D});
        return status(rpp::ops::tensor_to_lie(Strategy{}, {}, ob, ab, lie, bd.basis, n, m));
    }
    auto ob = rpp::make_tensor_batch(out, static_cast<Index>(out_stride), Degree{0}, Degree{D});
    auto ab = rpp::make_lie_batch(arg, static_cast<Index>(arg_stride), Degree{1}, Degree{D});
    return status(rpp::ops::lie_to_tensor(Strategy{}, {}, ob, ab, bd.basis, lie, n, m));
}

// Signature of a ragged batch of piecewise-linear paths by the caller loop
// of ft_fmexp (tests/rpp/gpu/block/ops/ft_fmexp_tests.cu:126-147): S_0 = 1,
// S_k = ft_fmexp(S_{k-1}, X_k) with X_k holding the increment in degree one.
// Paths are split over `threads` host threads, each issuing its own launches.
int ref_signature(int32_t W, int32_t D, int64_t n, double const* incr, int64_t const* offsets,
                  double* sig, int32_t threads) {
    BasisData bd(W, D);
    const Index dim = bd.basis.size();
    if (threads < 1) threads = 1;
    std::vector<int> rc(static_cast<size_t>(threads), 0);
    auto work = [&](int t, int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) {
            std::vector<double> cur(static_cast<size_t>(dim), 0.0), next(static_cast<size_t>(dim));
            std::vector<double> x(static_cast<size_t>(1 + W), 0.0);
            cur[0] = 1.0;
            for (int64_t k = offsets[b]; k < offsets[b + 1]; ++k) {
                std::memcpy(x.data() + 1, incr + k * W, sizeof(double) * static_cast<size_t>(W));
                auto ob = rpp::make_tensor_batch(next.data(), dim, Degree{0}, Degree{D});
                auto mb = rpp::make_tensor_batch(static_cast<double const*>(cur.data()), dim,
                                                 Degree{0}, Degree{D});
                auto xb = rpp::make_tensor_batch(static_cast<double const*>(x.data()),
                                                 static_cast<Index>(1 + W), Degree{1}, Degree{1});
                if (auto err = rpp::ops::ft_fmexp(Strategy{}, {}, ob, mb, xb, bd.basis, 1); !err) {
                    rc[static_cast<size_t>(t)] = 1 + static_cast<int>(err.code());
                    return;
                }
                cur.swap(next);
            }
            std::memcpy(sig + b * dim, cur.data(), sizeof(double) * static_cast<size_t>(dim));
        }
    };
    const int64_t per = (n + threads - 1) / threads;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const int64_t b0 = t * per, b1 = std::min<int64_t>(n, b0 + per);
        if (b0 >= b1) break;
        pool.emplace_back(work, t, b0, b1);
    }
    for (auto& th : pool) th.join();
    for (int r : rc)
        if (r) return r;
    return 0;
}

// Forward signature and the stored-prefix reverse pass of a ragged batch,
// each path by the reference's own operations (the CPU form of the
// per-operation composition a reference user writes for the gradient of
// loss = sum_b <ell_b, S(x_b)>):
//   forward   S_k = ft_fmexp(S_{k-1}, X_k), every prefix stored;
//   reverse   G_L = ell_b; for k = L..1:
//               E   = ft_exp(X_k)
//               H   = ft_adj_lmul(S_{k-1}, G_k)       (d loss / d E_k)
//               grad x_k = H contracted with dE_k/dx_k  (no reference op: the
//                          derivative of prod_i x[w_i] / |w|! in each letter)
//               G_{k-1} = ft_adj_rmul(E, G_k).
// X_k holds increment k in degree one.  `sig` (may be null) receives S_L.
// Paths are split over `threads` host threads, each issuing its own calls.
int ref_signature_grad(int32_t W, int32_t D, int64_t n, double const* incr, int64_t const* offsets,
                       double const* ell, double* sig, double* grad, int32_t threads) {
    BasisData bd(W, D);
    const Index dim = bd.basis.size();
    if (threads < 1) threads = 1;
    std::vector<int> rc(static_cast<size_t>(threads), 0);
    auto full = [&](double* p) { return rpp::make_tensor_batch(p, dim, Degree{0}, Degree{D}); };
    auto cfull = [&](double const* p) { return rpp::make_tensor_batch(p, dim, Degree{0}, Degree{D}); };
    auto work = [&](int t, int64_t b0, int64_t b1) {
        std::vector<double> G(static_cast<size_t>(dim)), Gn(static_cast<size_t>(dim)), H(static_cast<size_t>(dim)),
            E(static_cast<size_t>(dim)), x(static_cast<size_t>(1 + W), 0.0), before(static_cast<size_t>(D) + 1),
            after(static_cast<size_t>(D) + 1);
        std::vector<int> letters(static_cast<size_t>(D) + 1);
        std::vector<double> prefixes;
        auto fail = [&](auto const& err) {
            rc[static_cast<size_t>(t)] = 1 + static_cast<int>(err.code());
        };
        for (int64_t b = b0; b < b1; ++b) {
            const int64_t off = offsets[b], len = offsets[b + 1] - off;
            prefixes.assign(static_cast<size_t>(dim * (len + 1)), 0.0);
            prefixes[0] = 1.0;
            for (int64_t k = 0; k < len; ++k) {
                std::memcpy(x.data() + 1, incr + (off + k) * W, sizeof(double) * static_cast<size_t>(W));
                auto xb = rpp::make_tensor_batch(static_cast<double const*>(x.data()), static_cast<Index>(1 + W),
                                                 Degree{1}, Degree{1});
                if (auto err = rpp::ops::ft_fmexp(Strategy{}, {}, full(prefixes.data() + (k + 1) * dim),
                                                  cfull(prefixes.data() + k * dim), xb, bd.basis, 1);
                    !err) {
                    fail(err);
                    return;
                }
            }
            if (sig) std::memcpy(sig + b * dim, prefixes.data() + len * dim, sizeof(double) * static_cast<size_t>(dim));
            if (!grad) continue;
            std::memcpy(G.data(), ell + b * dim, sizeof(double) * static_cast<size_t>(dim));
            for (int64_t k = len - 1; k >= 0; --k) {
                double const* xk = incr + (off + k) * W;
                std::memcpy(x.data() + 1, xk, sizeof(double) * static_cast<size_t>(W));
                auto xb = rpp::make_tensor_batch(static_cast<double const*>(x.data()), static_cast<Index>(1 + W),
                                                 Degree{1}, Degree{1});
                if (auto err = rpp::ops::ft_exp(Strategy{}, {}, full(E.data()), xb, bd.basis, 1); !err) {
                    fail(err);
                    return;
                }
                if (auto err = rpp::ops::ft_adj_lmul(Strategy{}, {}, full(H.data()), cfull(prefixes.data() + k * dim),
                                                     cfull(G.data()), bd.basis, 1);
                    !err) {
                    fail(err);
                    return;
                }
                double* g = grad + (off + k) * W;
                for (int32_t a = 0; a < W; ++a) g[a] = 0.0;
                double fact = 1.0;
                Index begin = 1, width_n = 1;
                for (int32_t deg = 1; deg <= D; ++deg) {
                    fact *= deg;
                    width_n *= W;
                    for (Index i = 0; i < width_n; ++i) {
                        const double h = H[static_cast<size_t>(begin + i)];
                        if (h == 0.0) continue;
                        Index r = i;
                        for (int32_t p = deg - 1; p >= 0; --p) {
                            letters[static_cast<size_t>(p)] = static_cast<int>(r % W);
                            r /= W;
                        }
                        before[0] = 1.0;
                        for (int32_t p = 0; p < deg; ++p) before[p + 1] = before[p] * xk[letters[p]];
                        after[deg] = 1.0;
                        for (int32_t p = deg - 1; p >= 0; --p) after[p] = after[p + 1] * xk[letters[p]];
                        const double hs = h / fact;
                        for (int32_t p = 0; p < deg; ++p) g[letters[p]] += hs * before[p] * after[p + 1];
                    }
                    begin += width_n;
                }
                if (auto err = rpp::ops::ft_adj_rmul(Strategy{}, {}, full(Gn.data()), cfull(E.data()),
                                                     cfull(G.data()), bd.basis, 1);
                    !err) {
                    fail(err);
                    return;
                }
                G.swap(Gn);
            }
        }
    };
    const int64_t per = (n + threads - 1) / threads;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const int64_t b0 = t * per, b1 = std::min<int64_t>(n, b0 + per);
        if (b0 >= b1) break;
        pool.emplace_back(work, t, b0, b1);
    }
    for (auto& th : pool) th.join();
    for (int r : rc)
        if (r) return r;
    return 0;
}

// Shuffle algebra through the public front ends (include/rpp/operations/basic/
// st_mul.hpp, st_fma.hpp, st_inplace_fma.hpp, st_adj_mul.hpp, left_hs_mul.hpp,
// tensor_pairing.hpp).  mode 0: st_mul(out, b, c, beta); 1: st_fma(out, a, b,
// c, alpha, beta); 2: st_inplace_fma(out, b, c, alpha, beta).
int ref_st(int32_t W, int32_t D, int64_t n, int mode, Arg const* out, Arg const* a, Arg const* b,
           Arg const* c, double alpha, double beta) {
    BasisData bd(W, D);
    if (mode == 0)
        return status(rpp::ops::st_mul(Strategy{}, {}, batch(out), cbatch(b), cbatch(c), bd.basis, n, beta));
    if (mode == 1)
        return status(rpp::ops::st_fma(Strategy{}, {}, batch(out), cbatch(a), cbatch(b), cbatch(c), bd.basis,
                                       n, alpha, beta));
    return status(
        rpp::ops::st_inplace_fma(Strategy{}, {}, batch(out), cbatch(b), cbatch(c), bd.basis, n, alpha, beta));
}

int ref_st_adj_mul(int32_t W, int32_t D, int64_t n, Arg const* out, Arg const* op, Arg const* arg) {
    BasisData bd(W, D);
    return status(rpp::ops::st_adj_mul(Strategy{}, {}, batch(out), cbatch(op), cbatch(arg), bd.basis, n));
}

int ref_left_hs_mul(int32_t W, int32_t D, int64_t n, Arg const* out, Arg const* x, Arg const* y,
                    double beta) {
    BasisData bd(W, D);
    return status(rpp::ops::left_hs_mul(Strategy{}, {}, batch(out), cbatch(x), cbatch(y), bd.basis, n, beta));
}

// The CPU strategy's half-shuffle adjoints take no scale factor, so they are
// driven through their operation objects, as the reference's own tests do
// (tests/rpp/cpu/single_thread/ops/left_hs_adjoint_tests.cpp:29-56):
// (out, integrator, integrand) in the operator's argument order.
int ref_left_hs_adjoint(int32_t W, int32_t D, int64_t n, int lmul, Arg const* out, Arg const* integrator,
                        Arg const* integrand) {
    BasisData bd(W, D);
    const Strategy::Context ctx(nullptr);
    for (int64_t b = 0; b < n; ++b) {
        rpp::DenseTensorView<double*, Basis> o(out->data + b * out->stride, bd.basis, Degree{out->min_degree},
                                          Degree{out->max_degree});
        rpp::DenseTensorView<double const*, Basis> x(integrator->data + b * integrator->stride, bd.basis,
                                                Degree{integrator->min_degree}, Degree{integrator->max_degree});
        rpp::DenseTensorView<double const*, Basis> y(integrand->data + b * integrand->stride, bd.basis,
                                                Degree{integrand->min_degree}, Degree{integrand->max_degree});
        if (lmul)
            rpp::ops::LeftHSAdjLMul<Strategy>{ctx, rpp::basis::make_basis_pack(bd.basis)}(ctx, o, x, y);
        else
            rpp::ops::LeftHSAdjRMul<Strategy>{ctx, rpp::basis::make_basis_pack(bd.basis)}(ctx, o, x, y);
    }
    return 0;
}

int ref_tensor_pairing(int32_t W, int32_t D, int64_t n, double* result, Arg const* f, Arg const* a) {
    BasisData bd(W, D);
    return status(rpp::ops::tensor_pairing(Strategy{}, {}, rpp::make_scalar_batch(result), cbatch(f), cbatch(a),
                                           bd.basis, n));
}

}  // extern "C"
