// rpp/gpu/gb300/strategy.hpp -- the GB300 (sm_103a) execution strategy for
// RoughPathPrimitives' operation API.
//
// Drop-in for rpp::gpu::strategies::BlockStrategy
// (include/rpp/gpu/block/strategy.hpp:212-365): it exposes the same member
// types and the same `launch<Op>(LaunchConfig&&, Batches&&, Bases&&, Index,
// Extras...) -> Error<char const*>` entry point, so caller code written
// against rpp::ops::<op>(strategy, config, ...) compiles unchanged with
//     rpp::gpu::strategies::GB300Strategy<double> strategy;
// Every operation specialisation below forwards to the C ABI of
// include/rpp_gb300.h (librpp_gb300.so), whose kernels are hand-written for
// sm_103a.  Batch data must be device memory, as with BlockStrategy.
//
// Differences from BlockStrategy that a caller can observe:
//  * basis tables and sparse matrices are uploaded once and cached (plans /
//    matrix handles keyed by (width, depth, device) and by the host arrays),
//    where BlockStrategy re-uploads them on every launch
//    (include/rpp/gpu/device.hpp:176-209); nothing is allocated per launch,
//    so launches can be captured in CUDA graphs;
//  * sparse products use the CPU strategy's begin-relative indexing
//    (include/rpp/cpu/single_thread/operations/linalg/
//    sparse_matrix_vector.hpp) and CSC matrices are transposed to CSR once,
//    so results are deterministic (no atomics).
#ifndef RPP_GPU_GB300_STRATEGY_HPP
#define RPP_GPU_GB300_STRATEGY_HPP

#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include <rpp/config.h>
#include <rpp/gpu/architecture.hpp>
#include <rpp/gpu/device.hpp>
#include <rpp/operations.hpp>
#include <rpp/sparse/matrix.hpp>
#include <rpp/support/error.hpp>
#include <rpp/utility.hpp>

#include <rpp_gb300.h>

namespace rpp::gpu::strategies {

template <typename Accum_, typename Architecture_>
struct GB300Strategy;

namespace gb300_detail {

// Host-side context: operations of this strategy never run on the host or
// inside a generic kernel; the type exists for BaseOperation's typedefs.
template <typename Strategy_>
struct Context {
    using Strategy = Strategy_;
    using Index = typename Strategy::Index;
    using Degree = typename Strategy::Degree;
    using Accum = typename Strategy::Accum;
};

template <typename Accum>
constexpr int32_t dtype_code() noexcept {
    static_assert(std::is_same_v<Accum, float> || std::is_same_v<Accum, double>,
                  "GB300Strategy supports float and double accumulation");
    return std::is_same_v<Accum, double> ? RPP_GB_F64 : RPP_GB_F32;
}

inline Error<char const*> status(int rc) noexcept {
    if (rc == RPP_GB_SUCCESS) return Error<char const*>::success();
    return Error<char const*>(static_cast<ErrorCode>(rc), rpp_gb_last_error_string());
}

// Plans are immutable and shared; one per (width, depth, device).
inline Error<char const*> get_plan(int32_t width, int32_t depth, int32_t device,
                                   rpp_gb_plan const*& plan) noexcept {
    static std::mutex lock;
    static std::map<std::tuple<int32_t, int32_t, int32_t>, rpp_gb_plan*> plans;
    std::lock_guard<std::mutex> guard(lock);
    auto key = std::make_tuple(width, depth, device);
    auto it = plans.find(key);
    if (it == plans.end()) {
        rpp_gb_plan* p = nullptr;
        if (int rc = rpp_gb_plan_create(&p, width, depth, device); rc != RPP_GB_SUCCESS) return status(rc);
        it = plans.emplace(key, p).first;
    }
    plan = it->second;
    return Error<char const*>::success();
}

inline int32_t current_device() noexcept {
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

template <typename T>
auto raw(T ptr) noexcept {
    return raw_pointer_cast(ptr);
}

// {data, stride, degree range} of batch element 0, resolved through the
// basis pack exactly as the kernels of the reference resolve it
// (include/rpp/views/batch.hpp:139-144).
template <typename Batch, typename Bases>
rpp_gb_tensor_arg tensor_arg(Batch const& batch, Bases const& bases) noexcept {
    using Index = typename std::decay_t<Batch>::Index;
    auto view = batch.view(bases, Index{0});
    rpp_gb_tensor_arg a;
    a.data = const_cast<void*>(static_cast<void const*>(raw(view.data())));
    a.stride = static_cast<int64_t>(batch.layout().stride_);
    a.min_degree = static_cast<int32_t>(view.min_degree());
    a.max_degree = static_cast<int32_t>(view.max_degree());
    return a;
}

// Begin-relative vector operand of a sparse product.
template <typename Batch, typename Bases>
rpp_gb_vector_arg vector_arg(Batch const& batch, Bases const& bases) noexcept {
    using Index = typename std::decay_t<Batch>::Index;
    auto view = batch.view(bases, Index{0});
    rpp_gb_vector_arg a;
    a.data = const_cast<void*>(static_cast<void const*>(raw(view.data())));
    a.stride = static_cast<int64_t>(batch.layout().stride_);
    a.begin = static_cast<int64_t>(view.begin_index());
    a.size = static_cast<int64_t>(view.end_index() - view.begin_index());
    return a;
}

template <typename Batch, typename Bases>
auto const& batch_basis(Batch const& batch, Bases const& bases) noexcept {
    using Index = typename std::decay_t<Batch>::Index;
    return batch.view(bases, Index{0}).basis();
}

template <typename Batch>
using batch_scalar_t = std::remove_cv_t<std::remove_reference_t<decltype(*raw(std::declval<Batch const&>().data()))>>;

template <typename Accum, typename... Batches>
constexpr bool scalars_match() noexcept {
    return (std::is_same_v<batch_scalar_t<std::decay_t<Batches>>, Accum> && ...);
}

// Sparse matrices are uploaded once per (host arrays, device).
template <typename Matrix>
Error<char const*> get_matrix(Matrix const& m, int32_t device, rpp_gb_matrix const*& out) noexcept {
    static std::mutex lock;
    static std::map<std::tuple<void const*, void const*, void const*, int64_t, int32_t>, rpp_gb_matrix*> cache;
    std::lock_guard<std::mutex> guard(lock);
    auto key = std::make_tuple(static_cast<void const*>(raw(m.data())), static_cast<void const*>(raw(m.indices())),
                               static_cast<void const*>(raw(m.offsets())), static_cast<int64_t>(m.nnz()), device);
    auto it = cache.find(key);
    if (it == cache.end()) {
        const int64_t nnz = static_cast<int64_t>(m.nnz()), outer = static_cast<int64_t>(m.outer_dim());
        std::vector<int64_t> offsets(static_cast<size_t>(outer) + 1), indices(static_cast<size_t>(nnz));
        std::vector<double> values(static_cast<size_t>(nnz));
        for (int64_t i = 0; i <= outer; ++i) offsets[i] = static_cast<int64_t>(m.offset(i));
        for (int64_t i = 0; i < nnz; ++i) {
            indices[i] = static_cast<int64_t>(m.inner_index(i));
            values[i] = static_cast<double>(m.value(i));
        }
        constexpr int32_t fmt = Matrix::format == sparse::detail::CompressedFormat::CSR ? RPP_GB_CSR : RPP_GB_CSC;
        rpp_gb_matrix* h = nullptr;
        if (int rc = rpp_gb_matrix_create(&h, fmt, outer, static_cast<int64_t>(m.inner_dim()), nnz, offsets.data(),
                                          indices.data(), values.data(), device);
            rc != RPP_GB_SUCCESS)
            return status(rc);
        it = cache.emplace(key, h).first;
    }
    out = it->second;
    return Error<char const*>::success();
}

}  // namespace gb300_detail

template <typename Accum_, typename Architecture_ = arch::DefaultArchitecture>
struct GB300Strategy {
    using Accum = Accum_;
    using Architecture = Architecture_;
    using Size = typename Architecture::Size;
    using Index = typename Architecture::Index;
    using Letter = typename Architecture::Letter;
    using Bitmask = typename Architecture::Bitmask;
    using Degree = typename Architecture::Degree;
    using Context = gb300_detail::Context<GB300Strategy>;
    using LaunchConfig = DeviceLaunchConfig;

    // CUDA device the operations run on; -1 = the calling thread's current device.
    int32_t device = -1;

    int32_t device_id() const noexcept { return device >= 0 ? device : gb300_detail::current_device(); }

    // Same signature as BlockStrategy::launch (include/rpp/gpu/block/
    // strategy.hpp:295-300).  The operation's specialisation does the work.
    template <typename Op, typename Batches, typename Bases, typename... Extras>
    RPP_HOST Error<char const*> launch(LaunchConfig&& config, Batches&& batches, Bases&& bases, Index batch_size,
                                       Extras... extras) const noexcept {
        return Op::gb300_launch(*this, config, std::forward<Batches>(batches), std::forward<Bases>(bases),
                                batch_size, extras...);
    }
};

}  // namespace rpp::gpu::strategies

namespace rpp::ops {

#define RPP_GB300_OP_HEADER(NAME)                                                                             \
    template <typename Accum_, typename Architecture_>                                                       \
    class NAME<gpu::strategies::GB300Strategy<Accum_, Architecture_>>                                        \
        : public BaseOperation<gpu::strategies::GB300Strategy<Accum_, Architecture_>> {                      \
    public:                                                                                                   \
        using Strategy = gpu::strategies::GB300Strategy<Accum_, Architecture_>;                              \
        using Accum = Accum_;                                                                                 \
        using Index = typename Strategy::Index;                                                               \
        using BaseOperation<Strategy>::BaseOperation;                                                         \
        static constexpr bool is_implemented = true;

namespace gb300_ops_detail {

using gpu::strategies::gb300_detail::status;
using gpu::strategies::gb300_detail::tensor_arg;

template <typename Strategy, typename Basis>
Error<char const*> plan_of(Strategy const& s, Basis const& basis, rpp_gb_plan const*& plan) noexcept {
    return gpu::strategies::gb300_detail::get_plan(static_cast<int32_t>(basis.width),
                                                   static_cast<int32_t>(basis.depth), s.device_id(), plan);
}

template <typename Bases>
auto const& tensor_basis(Bases const& bases) noexcept {
    return basis::get_basis(basis::TensorBasisTag{}, bases);
}

}  // namespace gb300_ops_detail

// ---- ft_mul (include/rpp/operations/basic/ft_mul.hpp:48-79) ---------------
RPP_GB300_OP_HEADER(FTMul)
    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Accum beta = Accum{1}) noexcept {
        namespace d = gb300_ops_detail;
        static_assert(gpu::strategies::gb300_detail::scalars_match<Accum, std::tuple_element_t<0, std::decay_t<Batches>>>(),
                      "batch scalar type must equal the strategy's Accum");
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto o = d::tensor_arg(std::get<0>(b), bases), l = d::tensor_arg(std::get<1>(b), bases),
             r = d::tensor_arg(std::get<2>(b), bases);
        return d::status(rpp_gb_ft_mul(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o, &l,
                                       &r, static_cast<int64_t>(n), static_cast<double>(beta)));
    }
};

// ---- ft_fma (include/rpp/operations/basic/ft_fma.hpp:48-83) ---------------
RPP_GB300_OP_HEADER(FTFma)
    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Accum alpha = Accum{1},
                                           Accum beta = Accum{1}) noexcept {
        namespace d = gb300_ops_detail;
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto o = d::tensor_arg(std::get<0>(b), bases), x = d::tensor_arg(std::get<1>(b), bases),
             y = d::tensor_arg(std::get<2>(b), bases), z = d::tensor_arg(std::get<3>(b), bases);
        return d::status(rpp_gb_ft_fma(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o, &x,
                                       &y, &z, static_cast<int64_t>(n), static_cast<double>(alpha),
                                       static_cast<double>(beta)));
    }
};

// ---- ft_inplace_fma<kind> (include/rpp/operations/basic/ft_inplace_fma.hpp) -
template <typename Accum_, typename Architecture_, FTInplaceFMAType FMAType>
class FTInplaceFma<gpu::strategies::GB300Strategy<Accum_, Architecture_>, FMAType>
    : public BaseOperation<gpu::strategies::GB300Strategy<Accum_, Architecture_>> {
public:
    using Strategy = gpu::strategies::GB300Strategy<Accum_, Architecture_>;
    using Accum = Accum_;
    using Index = typename Strategy::Index;
    using BaseOperation<Strategy>::BaseOperation;
    static constexpr bool is_implemented = true;

    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Accum alpha = Accum{1},
                                           Accum beta = Accum{1}) noexcept {
        namespace d = gb300_ops_detail;
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto a = d::tensor_arg(std::get<0>(b), bases), x = d::tensor_arg(std::get<1>(b), bases),
             y = d::tensor_arg(std::get<2>(b), bases);
        constexpr int32_t kind = FMAType == FTInplaceFMAType::AEqualsBCPlusA   ? RPP_GB_A_EQUALS_BC_PLUS_A
                                 : FMAType == FTInplaceFMAType::AEqualsABPlusC ? RPP_GB_A_EQUALS_AB_PLUS_C
                                                                               : RPP_GB_A_EQUALS_BA_PLUS_C;
        return d::status(rpp_gb_ft_inplace_fma(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(),
                                               kind, &a, &x, &y, static_cast<int64_t>(n),
                                               static_cast<double>(alpha), static_cast<double>(beta)));
    }
};

// ---- ft_inplace_mul (include/rpp/operations/basic/ft_inplace_mul.hpp) ------
RPP_GB300_OP_HEADER(FTInplaceMul)
    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Accum beta = Accum{1}) noexcept {
        namespace d = gb300_ops_detail;
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto l = d::tensor_arg(std::get<0>(b), bases), r = d::tensor_arg(std::get<1>(b), bases);
        return d::status(rpp_gb_ft_inplace_mul(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(),
                                               &l, &r, static_cast<int64_t>(n), static_cast<double>(beta)));
    }
};

#define RPP_GB300_BINARY_OP(NAME, CALL)                                                                       \
    RPP_GB300_OP_HEADER(NAME)                                                                                 \
        template <typename Batches, typename Bases>                                                           \
        static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg,         \
                                               Batches&& b, Bases&& bases, Index n) noexcept {                \
            namespace d = gb300_ops_detail;                                                                   \
            rpp_gb_plan const* plan = nullptr;                                                                \
            if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;                           \
            auto o = d::tensor_arg(std::get<0>(b), bases), a = d::tensor_arg(std::get<1>(b), bases);          \
            return d::status(CALL(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o,  \
                                  &a, static_cast<int64_t>(n)));                                              \
        }                                                                                                     \
    };

#define RPP_GB300_TERNARY_OP(NAME, CALL)                                                                      \
    RPP_GB300_OP_HEADER(NAME)                                                                                 \
        template <typename Batches, typename Bases>                                                           \
        static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg,         \
                                               Batches&& b, Bases&& bases, Index n) noexcept {                \
            namespace d = gb300_ops_detail;                                                                   \
            rpp_gb_plan const* plan = nullptr;                                                                \
            if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;                           \
            auto o = d::tensor_arg(std::get<0>(b), bases), x = d::tensor_arg(std::get<1>(b), bases),          \
                 y = d::tensor_arg(std::get<2>(b), bases);                                                    \
            return d::status(CALL(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o,  \
                                  &x, &y, static_cast<int64_t>(n)));                                          \
        }                                                                                                     \
    };

// ft_exp / ft_log (include/rpp/operations/intermediate/ft_exp.hpp, ft_log.hpp)
RPP_GB300_BINARY_OP(FTExp, rpp_gb_ft_exp)
RPP_GB300_BINARY_OP(FTLog, rpp_gb_ft_log)
// ft_fmexp(out, multiplier, exponent) (include/rpp/operations/intermediate/ft_fmexp.hpp)
RPP_GB300_TERNARY_OP(FTFMExp, rpp_gb_ft_fmexp)
// ft_adj_lmul / ft_adj_rmul (include/rpp/operations/basic/ft_adj_lmul.hpp, ft_adj_rmul.hpp)
RPP_GB300_TERNARY_OP(FTAdjLMul, rpp_gb_ft_adj_lmul)
RPP_GB300_TERNARY_OP(FTAdjRMul, rpp_gb_ft_adj_rmul)
// vector_assign (include/rpp/operations/linalg/vector_assign.hpp)
RPP_GB300_BINARY_OP(VectorAssign, rpp_gb_vector_assign)

// ---- shuffle algebra (include/rpp/operations/basic/st_*.hpp, left_hs_*.hpp) -
#define RPP_GB300_SCALED_TERNARY_OP(NAME, CALL)                                                               \
    RPP_GB300_OP_HEADER(NAME)                                                                                 \
        template <typename Batches, typename Bases>                                                           \
        static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg,         \
                                               Batches&& b, Bases&& bases, Index n,                           \
                                               Accum beta = Accum{1}) noexcept {                              \
            namespace d = gb300_ops_detail;                                                                   \
            rpp_gb_plan const* plan = nullptr;                                                                \
            if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;                           \
            auto o = d::tensor_arg(std::get<0>(b), bases), x = d::tensor_arg(std::get<1>(b), bases),          \
                 y = d::tensor_arg(std::get<2>(b), bases);                                                    \
            return d::status(CALL(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o,  \
                                  &x, &y, static_cast<int64_t>(n), static_cast<double>(beta)));               \
        }                                                                                                     \
    };

// st_mul(out, lhs, rhs, beta) (st_mul.hpp:53-79)
RPP_GB300_SCALED_TERNARY_OP(STMul, rpp_gb_st_mul)
// left_hs_mul(out, integrator, integrand, beta) (left_hs_mul.hpp:59-87)
RPP_GB300_SCALED_TERNARY_OP(LeftHSMul, rpp_gb_left_hs_mul)
// left_hs_adj_lmul / left_hs_adj_rmul(out, op, arg, beta) (left_hs_adj_lmul.hpp:39-57,
// left_hs_adj_rmul.hpp:39-57)
RPP_GB300_SCALED_TERNARY_OP(LeftHSAdjLMul, rpp_gb_left_hs_adj_lmul)
RPP_GB300_SCALED_TERNARY_OP(LeftHSAdjRMul, rpp_gb_left_hs_adj_rmul)
// st_adj_mul(out, op, arg) (st_adj_mul.hpp:46-69)
RPP_GB300_TERNARY_OP(STAdjMul, rpp_gb_st_adj_mul)

// ---- st_fma (st_fma.hpp:56-85) ----------------------------------------------
RPP_GB300_OP_HEADER(STFma)
    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Accum alpha = Accum{1},
                                           Accum beta = Accum{1}) noexcept {
        namespace d = gb300_ops_detail;
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto o = d::tensor_arg(std::get<0>(b), bases), x = d::tensor_arg(std::get<1>(b), bases),
             y = d::tensor_arg(std::get<2>(b), bases), z = d::tensor_arg(std::get<3>(b), bases);
        return d::status(rpp_gb_st_fma(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o, &x,
                                       &y, &z, static_cast<int64_t>(n), static_cast<double>(alpha),
                                       static_cast<double>(beta)));
    }
};

// ---- st_inplace_fma (st_inplace_fma.hpp:50-80) ------------------------------
RPP_GB300_OP_HEADER(STInplaceFma)
    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Accum alpha = Accum{1},
                                           Accum beta = Accum{1}) noexcept {
        namespace d = gb300_ops_detail;
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto a = d::tensor_arg(std::get<0>(b), bases), x = d::tensor_arg(std::get<1>(b), bases),
             y = d::tensor_arg(std::get<2>(b), bases);
        return d::status(rpp_gb_st_inplace_fma(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(),
                                               &a, &x, &y, static_cast<int64_t>(n), static_cast<double>(alpha),
                                               static_cast<double>(beta)));
    }
};

// ---- tensor_pairing(result, functional, arg) (tensor_pairing.hpp:47-73) -----
// `result` is a scalar batch (rpp::make_scalar_batch) over a device array.
RPP_GB300_OP_HEADER(TensorPairing)
    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n) noexcept {
        namespace d = gb300_ops_detail;
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto f = d::tensor_arg(std::get<1>(b), bases), x = d::tensor_arg(std::get<2>(b), bases);
        void* result = const_cast<void*>(
            static_cast<void const*>(gpu::strategies::gb300_detail::raw(std::get<0>(b).data())));
        return d::status(rpp_gb_tensor_pairing(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(),
                                               result, &f, &x, static_cast<int64_t>(n)));
    }
};

// ---- tensor_generalised_antipode<policy> ---------------------------------
template <typename Accum_, typename Architecture_, TensorAntipodeSigningPolicy Policy>
class TensorGeneralisedAntipode<gpu::strategies::GB300Strategy<Accum_, Architecture_>, Policy>
    : public BaseOperation<gpu::strategies::GB300Strategy<Accum_, Architecture_>> {
public:
    using Strategy = gpu::strategies::GB300Strategy<Accum_, Architecture_>;
    using Accum = Accum_;
    using Index = typename Strategy::Index;
    using BaseOperation<Strategy>::BaseOperation;
    static constexpr bool is_implemented = true;

    template <typename Batches, typename Bases>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n) noexcept {
        namespace d = gb300_ops_detail;
        rpp_gb_plan const* plan = nullptr;
        if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;
        auto o = d::tensor_arg(std::get<0>(b), bases), a = d::tensor_arg(std::get<1>(b), bases);
        constexpr int32_t policy =
            Policy == TensorAntipodeSigningPolicy::SignByDegree ? RPP_GB_SIGN_BY_DEGREE : RPP_GB_NO_SIGNING;
        return d::status(rpp_gb_tensor_antipode(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(),
                                                policy, &o, &a, static_cast<int64_t>(n)));
    }
};

// ---- vector_set_constant / tensor_set_identity / tensor_add_identity ------
#define RPP_GB300_FILL_OP(NAME, CALL, DEFAULT)                                                                \
    RPP_GB300_OP_HEADER(NAME)                                                                                 \
        template <typename Batches, typename Bases>                                                           \
        static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg,         \
                                               Batches&& b, Bases&& bases, Index n,                           \
                                               Accum value = Accum{DEFAULT}) noexcept {                       \
            namespace d = gb300_ops_detail;                                                                   \
            rpp_gb_plan const* plan = nullptr;                                                                \
            if (auto e = d::plan_of(s, d::tensor_basis(bases), plan); !e) return e;                           \
            auto o = d::tensor_arg(std::get<0>(b), bases);                                                    \
            return d::status(CALL(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o,  \
                                  static_cast<int64_t>(n), static_cast<double>(value)));                      \
        }                                                                                                     \
    };

RPP_GB300_FILL_OP(VectorSetConstant, rpp_gb_vector_set_constant, 0)
RPP_GB300_FILL_OP(TensorSetIdentity, rpp_gb_tensor_set_identity, 1)
RPP_GB300_FILL_OP(TensorAddIdentity, rpp_gb_tensor_add_identity, 1)

// ---- sparse_matrix_vector_product<format> and the Lie conversions ---------
namespace gb300_ops_detail {

template <typename Strategy, typename Batches, typename Bases, typename Matrix>
Error<char const*> spmv(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches const& b, Bases const& bases,
                        typename Strategy::Index n, Matrix const& matrix, typename Strategy::Accum alpha) noexcept {
    rpp_gb_matrix const* m = nullptr;
    if (auto e = gpu::strategies::gb300_detail::get_matrix(matrix, s.device_id(), m); !e) return e;
    auto o = gpu::strategies::gb300_detail::vector_arg(std::get<0>(b), bases);
    auto a = gpu::strategies::gb300_detail::vector_arg(std::get<1>(b), bases);
    return status(rpp_gb_sparse_matrix_vector(m, cfg.stream,
                                              gpu::strategies::gb300_detail::dtype_code<typename Strategy::Accum>(),
                                              &o, &a, static_cast<int64_t>(n), static_cast<double>(alpha)));
}

}  // namespace gb300_ops_detail

template <typename Accum_, typename Architecture_, sparse::MatrixFormat Format>
class SparseMatrixVectorProduct<gpu::strategies::GB300Strategy<Accum_, Architecture_>, Format>
    : public BaseOperation<gpu::strategies::GB300Strategy<Accum_, Architecture_>> {
public:
    using Strategy = gpu::strategies::GB300Strategy<Accum_, Architecture_>;
    using Accum = Accum_;
    using Index = typename Strategy::Index;
    using BaseOperation<Strategy>::BaseOperation;
    static constexpr bool is_implemented = true;

    template <typename Batches, typename Bases, typename Matrix>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Matrix const& matrix,
                                           Accum alpha = Accum{1}) noexcept {
        return gb300_ops_detail::spmv(s, cfg, b, bases, n, matrix, alpha);
    }
};

template <typename Accum_, typename Architecture_, T2LImplementationType Impl>
class TensorToLie<gpu::strategies::GB300Strategy<Accum_, Architecture_>, Impl>
    : public BaseOperation<gpu::strategies::GB300Strategy<Accum_, Architecture_>> {
public:
    using Strategy = gpu::strategies::GB300Strategy<Accum_, Architecture_>;
    using Accum = Accum_;
    using Index = typename Strategy::Index;
    using BaseOperation<Strategy>::BaseOperation;
    static constexpr bool is_implemented = true;

    template <typename Batches, typename Bases, typename Matrix>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Matrix const& matrix) noexcept {
        return gb300_ops_detail::spmv(s, cfg, b, bases, n, matrix, Accum{1});
    }
};

template <typename Accum_, typename Architecture_, L2TImplementationType Impl>
class LieToTensor<gpu::strategies::GB300Strategy<Accum_, Architecture_>, Impl>
    : public BaseOperation<gpu::strategies::GB300Strategy<Accum_, Architecture_>> {
public:
    using Strategy = gpu::strategies::GB300Strategy<Accum_, Architecture_>;
    using Accum = Accum_;
    using Index = typename Strategy::Index;
    using BaseOperation<Strategy>::BaseOperation;
    static constexpr bool is_implemented = true;

    template <typename Batches, typename Bases, typename Matrix>
    static Error<char const*> gb300_launch(Strategy const& s, gpu::DeviceLaunchConfig const& cfg, Batches&& b,
                                           Bases&& bases, Index n, Matrix const& matrix) noexcept {
        return gb300_ops_detail::spmv(s, cfg, b, bases, n, matrix, Accum{1});
    }
};

#undef RPP_GB300_FILL_OP
#undef RPP_GB300_TERNARY_OP
#undef RPP_GB300_BINARY_OP
#undef RPP_GB300_OP_HEADER

// ---- signatures (new entry points; no reference operation) -----------------
// Signatures of a batch of piecewise-linear paths and, with seeds, the
// gradient of sum_b <seed_b, S(x_b)> in the same launch (rpp_gb_signature).
template <typename Accum, typename Architecture, typename Basis>
Error<char const*> signature(gpu::strategies::GB300Strategy<Accum, Architecture> const& s,
                             gpu::DeviceLaunchConfig const& cfg, Basis const& basis, Accum const* increments,
                             int64_t const* offsets, int64_t length, int64_t num_paths, Accum* sig,
                             int64_t sig_stride, Accum const* seed = nullptr, int64_t seed_stride = 0,
                             Accum* grad = nullptr) noexcept {
    rpp_gb_plan const* plan = nullptr;
    if (auto e = gb300_ops_detail::plan_of(s, basis, plan); !e) return e;
    return gb300_ops_detail::status(rpp_gb_signature(plan, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(),
                                                     increments, offsets, length, num_paths, sig, sig_stride, seed,
                                                     seed_stride, grad));
}

// ---- fused steps either side of the signature (no single reference call) ---
// tensor_log_to_lie: ft_log of `arg` over its own degree range, then
// tensor_to_lie of that log (include/rpp/operations/intermediate/ft_log.hpp,
// include/rpp/operations/basic/tensor_to_lie.hpp) in one kernel
// (rpp_gb_log_to_lie); `out` is a Lie batch.
template <typename Accum, typename Architecture, typename LieBatch, typename TensorBatch, typename LieBasis,
          typename TensorBasis, typename Matrix>
Error<char const*> tensor_log_to_lie(gpu::strategies::GB300Strategy<Accum, Architecture> const& s,
                                     gpu::DeviceLaunchConfig const& cfg, LieBatch const& out, TensorBatch const& arg,
                                     LieBasis const& lie_basis, TensorBasis const& tensor_basis,
                                     typename Architecture::Index n, Matrix const& matrix,
                                     Accum alpha = Accum{1}) noexcept {
    rpp_gb_plan const* plan = nullptr;
    if (auto e = gb300_ops_detail::plan_of(s, tensor_basis, plan); !e) return e;
    rpp_gb_matrix const* m = nullptr;
    if (auto e = gpu::strategies::gb300_detail::get_matrix(matrix, s.device_id(), m); !e) return e;
    auto bases = basis::make_basis_pack(lie_basis, tensor_basis);
    auto o = gpu::strategies::gb300_detail::vector_arg(out, bases);
    auto a = gpu::strategies::gb300_detail::tensor_arg(arg, bases);
    return gb300_ops_detail::status(rpp_gb_log_to_lie(plan, m, cfg.stream,
                                                      gpu::strategies::gb300_detail::dtype_code<Accum>(), &o, &a,
                                                      a.min_degree, a.max_degree, static_cast<int64_t>(n),
                                                      static_cast<double>(alpha)));
}

// lie_to_tensor_exp: lie_to_tensor of `arg` into out's degree range of a zero
// tensor X, then out = exp(X) (include/rpp/operations/basic/lie_to_tensor.hpp,
// include/rpp/operations/intermediate/ft_exp.hpp) in one kernel
// (rpp_gb_lie_to_tensor_exp); the overload with a multiplier batch computes
// out = multiplier (x) exp(X) (ft_fmexp.hpp).
template <typename Accum, typename Architecture, typename TensorBatch, typename LieBatch, typename TensorBasis,
          typename LieBasis, typename Matrix>
Error<char const*> lie_to_tensor_exp(gpu::strategies::GB300Strategy<Accum, Architecture> const& s,
                                     gpu::DeviceLaunchConfig const& cfg, TensorBatch const& out,
                                     TensorBatch const* multiplier, LieBatch const& arg,
                                     TensorBasis const& tensor_basis, LieBasis const& lie_basis,
                                     typename Architecture::Index n, Matrix const& matrix,
                                     Accum alpha = Accum{1}) noexcept {
    rpp_gb_plan const* plan = nullptr;
    if (auto e = gb300_ops_detail::plan_of(s, tensor_basis, plan); !e) return e;
    rpp_gb_matrix const* m = nullptr;
    if (auto e = gpu::strategies::gb300_detail::get_matrix(matrix, s.device_id(), m); !e) return e;
    auto bases = basis::make_basis_pack(tensor_basis, lie_basis);
    auto o = gpu::strategies::gb300_detail::tensor_arg(out, bases);
    auto a = gpu::strategies::gb300_detail::vector_arg(arg, bases);
    rpp_gb_tensor_arg mm{};
    if (multiplier) mm = gpu::strategies::gb300_detail::tensor_arg(*multiplier, bases);
    return gb300_ops_detail::status(rpp_gb_lie_to_tensor_exp(
        plan, m, cfg.stream, gpu::strategies::gb300_detail::dtype_code<Accum>(), &o, multiplier ? &mm : nullptr, &a,
        o.min_degree, o.max_degree, static_cast<int64_t>(n), static_cast<double>(alpha)));
}

}  // namespace rpp::ops

#endif  // RPP_GPU_GB300_STRATEGY_HPP
