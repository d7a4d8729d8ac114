// Drives the reference's own operation front ends (rpp::ops::<op>) with the
// GB300Strategy and prints the C-ABI calls they produce (recorded by the
// mock library).  Built and checked by tests/test_strategy_header.py.
#include <cstdio>
#include <string>
#include <vector>

#include <rpp/basis/hall_basis.hpp>
#include <rpp/basis/lie_multiplication.hpp>
#include <rpp/basis/tensor_basis.hpp>
#include <rpp/gpu/gb300/strategy.hpp>
#include <rpp/sparse/l2t_matrix.hpp>
#include <rpp/sparse/t2l_matrix.hpp>
#include <rpp/views/views.hpp>

extern std::string g_calls;

int main() {
    using Strategy = rpp::gpu::strategies::GB300Strategy<double>;
    using Arch = rpp::arch::NativeArchitecture;
    using Index = Arch::Index;
    using Degree = Arch::Degree;
    const Degree W = 3, D = 4;
    std::vector<Index> db{0, 1, 4, 13, 40, 121};
    rpp::basis::TensorBasis<Arch> basis(W, D, db.data());
    Strategy s{2};
    rpp::gpu::DeviceLaunchConfig cfg{nullptr, {}};
    std::vector<double> buf(4 * 128);
    double* p = buf.data();
    auto full = rpp::make_tensor_batch(p, Index{128}, Degree{0}, D);
    auto part = rpp::make_tensor_batch(p, Index{128}, Degree{1}, Degree{2});
    auto one = rpp::make_tensor_batch(p, Index{121}, Degree{1}, Degree{1});
    int bad = 0;
    bad += !rpp::ops::ft_mul(s, cfg, full, part, one, basis, 4, 0.5);
    bad += !rpp::ops::ft_fma(s, cfg, full, part, full, one, basis, 4, 0.25, 2.0);
    bad += !rpp::ops::ft_inplace_fma<rpp::ops::FTInplaceFMAType::AEqualsABPlusC>(s, cfg, full, one, part, basis, 4,
                                                                                  1.0, 0.5);
    bad += !rpp::ops::ft_inplace_mul(s, cfg, full, one, basis, 4, 3.0);
    bad += !rpp::ops::ft_exp(s, cfg, full, part, basis, 4);
    bad += !rpp::ops::ft_fmexp(s, cfg, full, part, one, basis, 4);
    bad += !rpp::ops::ft_log(s, cfg, full, part, basis, 4);
    bad += !rpp::ops::ft_adj_lmul(s, cfg, part, full, one, basis, 4);
    bad += !rpp::ops::ft_adj_rmul(s, cfg, part, full, one, basis, 4);
    bad += !rpp::ops::tensor_antipode(s, cfg, full, part, basis, 4);
    bad += !rpp::ops::tensor_reflect(s, cfg, full, part, basis, 4);
    bad += !rpp::ops::st_mul(s, cfg, full, part, one, basis, 4, 0.5);
    bad += !rpp::ops::st_fma(s, cfg, full, part, full, one, basis, 4, 0.25, 2.0);
    bad += !rpp::ops::st_inplace_fma(s, cfg, full, one, part, basis, 4, 1.0, 0.5);
    bad += !rpp::ops::st_adj_mul(s, cfg, part, full, one, basis, 4);
    bad += !rpp::ops::left_hs_mul(s, cfg, full, part, one, basis, 4, 3.0);
    bad += !rpp::ops::left_hs_adj_lmul(s, cfg, part, full, one, basis, 4);
    bad += !rpp::ops::left_hs_adj_rmul(s, cfg, part, full, one, basis, 4, 2.0);
    std::vector<double> scalars(4);
    bad += !rpp::ops::tensor_pairing(s, cfg, rpp::make_scalar_batch(scalars.data()), part, one, basis, 4);

    rpp::basis::HallBasis<Arch> hall(W, D);
    auto lie = hall.to_lie_basis();
    rpp::basis::LieMultiplicationCache<Arch> cache(lie);
    auto t2l = rpp::sparse::make_t2l_matrix<double>(lie, cache);
    using M = rpp::sparse::GradedMatrixView<rpp::sparse::MatrixFormat::CSC, double const*, Index const*, Index const*>;
    M m(t2l.data(), t2l.indices(), t2l.offsets(), t2l.nnz(), t2l.outer_dim(), t2l.inner_dim());
    std::vector<double> lbuf(4 * 40);
    auto lie_out = rpp::make_lie_batch(lbuf.data(), Index{40}, Degree{1}, D);
    auto tens_in = rpp::make_tensor_batch(static_cast<double const*>(p), Index{128}, Degree{0}, D);
    bad += !rpp::ops::tensor_to_lie(s, cfg, lie_out, tens_in, lie, basis, 4, m);
    bad += !rpp::ops::tensor_to_lie(s, cfg, lie_out, tens_in, lie, basis, 4, m);  // matrix cached: no new upload
    bad += !rpp::ops::signature(s, cfg, basis, p, static_cast<int64_t const*>(nullptr), 16, 4, p, 121);
    bad += !rpp::ops::tensor_log_to_lie(s, cfg, lie_out, tens_in, lie, basis, 4, m, 0.5);
    auto l2t = rpp::sparse::make_l2t_matrix<double>(lie);
    M ml(l2t.data(), l2t.indices(), l2t.offsets(), l2t.nnz(), l2t.outer_dim(), l2t.inner_dim());
    auto lie_in = rpp::make_lie_batch(static_cast<double const*>(lbuf.data()), Index{40}, Degree{1}, D);
    bad += !rpp::ops::lie_to_tensor_exp(s, cfg, full, static_cast<decltype(full) const*>(nullptr), lie_in, basis, lie,
                                        4, ml);
    bad += !rpp::ops::lie_to_tensor_exp(s, cfg, full, &full, lie_in, basis, lie, 4, ml, 2.0);
    std::fputs(g_calls.c_str(), stdout);
    std::printf("failures=%d\n", bad);
    return bad;
}
