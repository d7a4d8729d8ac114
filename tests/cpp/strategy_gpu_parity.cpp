// Runs the reference's own operation front ends (rpp::ops::<op>) twice on the
// same seeded inputs: with GB300Strategy on device buffers (the kernels of
// librpp_gb300.so) and with the reference's CPU SingleThreadStrategy on host
// copies, then prints one line per call with the largest relative difference
// |a - e| / max(1, |a|, |e|) over the output batch (the reference's metric,
// tests/rpp/cpu/single_thread/ops/cpu_typed_ft_ops_test_helper.hpp:261-273).
// The calls are the ones a reference user writes; only the strategy type
// differs.  Built and checked by tests/test_strategy_gpu.py.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <random>
#include <string>
#include <vector>

#include <rpp/basis/hall_basis.hpp>
#include <rpp/basis/lie_multiplication.hpp>
#include <rpp/basis/tensor_basis.hpp>
#include <rpp/cpu/single_thread/operations.hpp>
#include <rpp/cpu/strategies.hpp>
#include <rpp/gpu/gb300/strategy.hpp>
#include <rpp/sparse/l2t_matrix.hpp>
#include <rpp/sparse/t2l_matrix.hpp>
#include <rpp/views/views.hpp>

namespace {

using Arch = rpp::arch::NativeArchitecture;
using Index = Arch::Index;
using Degree = Arch::Degree;
using Gpu = rpp::gpu::strategies::GB300Strategy<double>;
using Cpu = rpp::cpu::strategies::SingleThreadStrategy<double>;

constexpr Degree W = 3, D = 4;
constexpr Index kDim = 121, kStride = 128, kN = 6;
constexpr Index kLieStride = 40;  // Hall basis W3 D4: 32 elements + the unused slot 0

int failures = 0;

// A batch held on both sides: `h` on the host (the CPU strategy's operand)
// and `d` on the device (GB300Strategy's).
struct Buf {
    std::vector<double> h;
    double* d = nullptr;
    explicit Buf(size_t n) : h(n, 0.0) {
        if (cudaMalloc(&d, n * sizeof(double)) != cudaSuccess) {
            std::printf("cudaMalloc failed\n");
            std::exit(2);
        }
    }
    ~Buf() { cudaFree(d); }
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    void fill(std::mt19937_64& rng) {
        std::uniform_real_distribution<double> u(-1.0, 1.0);
        for (auto& v : h) v = u(rng);
        push();
    }
    void push() { cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice); }
    std::vector<double> pull() const {
        std::vector<double> out(h.size());
        cudaMemcpy(out.data(), d, h.size() * sizeof(double), cudaMemcpyDeviceToHost);
        return out;
    }
};

double rel_diff(const std::vector<double>& a, const std::vector<double>& e) {
    double worst = 0.0;
    for (size_t i = 0; i < a.size(); ++i) {
        const double scale = std::max({1.0, std::abs(a[i]), std::abs(e[i])});
        const double d = std::abs(a[i] - e[i]) / scale;
        if (!(d <= worst)) worst = d;  // NaN counts as worst
    }
    return worst;
}

// Runs one operation on both strategies and reports it.  `run(gpu)` issues
// the call on the strategy named by `gpu`; `out` is the output buffer, whose
// host side holds the CPU result afterwards and whose device side the GPU's.
template <typename Run>
void check(const char* name, Buf& out, Run run) {
    out.push();  // both sides start from the same output contents (in-place kinds read them)
    const bool ok_cpu = run(false);
    const bool ok_gpu = run(true);
    const cudaError_t sync = cudaDeviceSynchronize();
    if (!ok_cpu || !ok_gpu || sync != cudaSuccess) {
        std::printf("%s status cpu=%d gpu=%d sync=%d\n", name, ok_cpu, ok_gpu, static_cast<int>(sync));
        ++failures;
        return;
    }
    std::printf("%s %.3e\n", name, rel_diff(out.pull(), out.h));
}

}  // namespace

int main() {
    std::vector<Index> db{0, 1, 4, 13, 40, 121};
    rpp::basis::TensorBasis<Arch> basis(W, D, db.data());
    Gpu gpu{0};
    Cpu cpu{};
    rpp::gpu::DeviceLaunchConfig gcfg{nullptr, {}};
    std::mt19937_64 rng(20240531);

    Buf a(kN * kStride), b(kN * kStride), c(kN * kStride), out(kN * kStride);
    a.fill(rng);
    b.fill(rng);
    c.fill(rng);
    out.fill(rng);
    auto T = [&](Buf& buf, bool dev, Degree lo, Degree hi) {
        return rpp::make_tensor_batch(dev ? buf.d : buf.h.data(), kStride, lo, hi);
    };
    auto C = [&](Buf& buf, bool dev, Degree lo, Degree hi) {
        return rpp::make_tensor_batch(static_cast<double const*>(dev ? buf.d : buf.h.data()), kStride, lo, hi);
    };
    // `call(op)` runs the front end on the chosen strategy with its own config
    auto call = [&](bool dev, auto&& op) -> bool {
        if (dev) return static_cast<bool>(op(gpu, rpp::gpu::DeviceLaunchConfig{gcfg}));
        return static_cast<bool>(op(cpu, typename Cpu::LaunchConfig{}));
    };

    check("ft_mul", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_mul(s, std::move(cfg), T(out, g, 0, D), C(a, g, 1, 2), C(b, g, 0, 3), basis, kN, 0.5);
        });
    });
    check("ft_fma", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_fma(s, std::move(cfg), T(out, g, 0, D), C(a, g, 0, D), C(b, g, 1, 3), C(c, g, 0, 2),
                                    basis, kN, 0.25, 2.0);
        });
    });
    check("ft_inplace_fma_abc", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_inplace_fma<rpp::ops::FTInplaceFMAType::AEqualsABPlusC>(
                s, std::move(cfg), T(out, g, 0, D), C(b, g, 0, D), C(c, g, 1, 2), basis, kN, 1.0, 0.5);
        });
    });
    check("ft_inplace_fma_bca", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_inplace_fma<rpp::ops::FTInplaceFMAType::AEqualsBCPlusA>(
                s, std::move(cfg), T(out, g, 0, D), C(b, g, 0, D), C(c, g, 0, D), basis, kN, 1.0, 1.0);
        });
    });
    check("ft_inplace_mul", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_inplace_mul(s, std::move(cfg), T(out, g, 0, D), C(b, g, 0, D), basis, kN, 3.0);
        });
    });
    check("ft_exp", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_exp(s, std::move(cfg), T(out, g, 0, D), C(a, g, 1, D), basis, kN);
        });
    });
    check("ft_fmexp", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_fmexp(s, std::move(cfg), T(out, g, 0, D), C(b, g, 0, D), C(a, g, 1, D), basis, kN);
        });
    });
    {
        // ft_log of tensors with unit scalar part
        Buf lg(kN * kStride);
        lg.h = a.h;
        for (Index k = 0; k < kN; ++k) lg.h[k * kStride] = 1.0;
        lg.push();
        check("ft_log", out, [&](bool g) {
            return call(g, [&](auto& s, auto cfg) {
                return rpp::ops::ft_log(s, std::move(cfg), T(out, g, 0, D), C(lg, g, 0, D), basis, kN);
            });
        });
    }
    check("ft_adj_lmul", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_adj_lmul(s, std::move(cfg), T(out, g, 0, D), C(a, g, 0, D), C(b, g, 0, D), basis, kN);
        });
    });
    check("ft_adj_rmul", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::ft_adj_rmul(s, std::move(cfg), T(out, g, 1, 3), C(a, g, 0, D), C(b, g, 0, D), basis, kN);
        });
    });
    check("tensor_antipode", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::tensor_antipode(s, std::move(cfg), T(out, g, 0, D), C(a, g, 0, D), basis, kN);
        });
    });
    check("tensor_reflect", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::tensor_reflect(s, std::move(cfg), T(out, g, 0, D), C(b, g, 1, 3), basis, kN);
        });
    });
    check("st_mul", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::st_mul(s, std::move(cfg), T(out, g, 0, D), C(a, g, 0, D), C(b, g, 0, D), basis, kN, 0.5);
        });
    });
    check("st_adj_mul", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::st_adj_mul(s, std::move(cfg), T(out, g, 0, D), C(a, g, 0, D), C(b, g, 0, D), basis, kN);
        });
    });
    check("left_hs_mul", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            return rpp::ops::left_hs_mul(s, std::move(cfg), T(out, g, 0, D), C(a, g, 1, D), C(b, g, 1, D), basis, kN,
                                         1.0);
        });
    });
    {
        Buf pair(kN);
        check("tensor_pairing", pair, [&](bool g) {
            return call(g, [&](auto& s, auto cfg) {
                double* r = g ? pair.d : pair.h.data();
                return rpp::ops::tensor_pairing(s, std::move(cfg), rpp::make_scalar_batch(r), C(a, g, 0, D),
                                                C(b, g, 0, D), basis, kN);
            });
        });
    }

    // Lie conversions through the reference's own generated matrices
    rpp::basis::HallBasis<Arch> hall(W, D);
    auto lie = hall.to_lie_basis();
    rpp::basis::LieMultiplicationCache<Arch> cache(lie);
    auto t2l = rpp::sparse::make_t2l_matrix<double>(lie, cache);
    auto l2t = rpp::sparse::make_l2t_matrix<double>(lie);
    using M = rpp::sparse::GradedMatrixView<rpp::sparse::MatrixFormat::CSC, double const*, Index const*, Index const*>;
    M mt(t2l.data(), t2l.indices(), t2l.offsets(), t2l.nnz(), t2l.outer_dim(), t2l.inner_dim());
    M ml(l2t.data(), l2t.indices(), l2t.offsets(), l2t.nnz(), l2t.outer_dim(), l2t.inner_dim());
    Buf lie_buf(kN * kLieStride);
    lie_buf.fill(rng);
    check("tensor_to_lie", lie_buf, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            auto lo = rpp::make_lie_batch(g ? lie_buf.d : lie_buf.h.data(), kLieStride, Degree{1}, D);
            return rpp::ops::tensor_to_lie(s, std::move(cfg), lo, C(a, g, 0, D), lie, basis, kN, mt);
        });
    });
    Buf lie_in(kN * kLieStride);
    lie_in.fill(rng);
    check("lie_to_tensor", out, [&](bool g) {
        return call(g, [&](auto& s, auto cfg) {
            auto li = rpp::make_lie_batch(static_cast<double const*>(g ? lie_in.d : lie_in.h.data()), kLieStride,
                                          Degree{1}, D);
            return rpp::ops::lie_to_tensor(s, std::move(cfg), T(out, g, 0, D), li, basis, lie, kN, ml);
        });
    });

    // Signatures: the new entry point on the GPU against the reference's
    // caller loop of ft_fmexp on the CPU strategy (ping-pong buffers: out must
    // not alias the multiplier).
    {
        const int64_t L = 24;
        std::normal_distribution<double> nd(0.0, 1.0 / std::sqrt(static_cast<double>(L)));
        Buf incr(kN * L * W), sig(kN * kDim);
        for (auto& v : incr.h) v = nd(rng);
        incr.push();
        check("signature", sig, [&](bool g) {
            if (g)
                return static_cast<bool>(rpp::ops::signature(gpu, gcfg, basis, incr.d, nullptr, L, kN, sig.d, kDim));
            std::vector<double> cur(kDim), next(kDim), x(1 + W, 0.0);
            for (Index p = 0; p < kN; ++p) {
                std::fill(cur.begin(), cur.end(), 0.0);
                cur[0] = 1.0;
                for (int64_t k = 0; k < L; ++k) {
                    std::copy_n(incr.h.data() + (p * L + k) * W, W, x.data() + 1);
                    auto ob = rpp::make_tensor_batch(next.data(), kDim, Degree{0}, D);
                    auto mb = rpp::make_tensor_batch(static_cast<double const*>(cur.data()), kDim, Degree{0}, D);
                    auto xb = rpp::make_tensor_batch(static_cast<double const*>(x.data()), Index{1 + W}, Degree{1},
                                                     Degree{1});
                    if (!rpp::ops::ft_fmexp(cpu, {}, ob, mb, xb, basis, 1)) return false;
                    cur.swap(next);
                }
                std::copy(cur.begin(), cur.end(), sig.h.begin() + p * kDim);
            }
            return true;
        });
    }
    std::printf("failures=%d\n", failures);
    return failures;
}
