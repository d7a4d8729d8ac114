// The reference's own GPU strategy (rpp::gpu::strategies::BlockStrategy),
// compiled unmodified from its headers for sm_103a and exposed through a few
// extern "C" wrappers, so that bench.py can drive the reference's plain
// per-operation GPU path -- the caller's loop of one ft_fmexp launch per
// increment (tests/rpp/gpu/block/ops/ft_fmexp_tests.cu:126-147) and, for the
// reverse pass, ft_exp / ft_adj_lmul / ft_adj_rmul per increment -- on the
// same device buffers as this repository's kernels.  This is a comparator, not
// part of the library: it is built only where the reference's headers are
// installed (baseline/_ref, or RPP_REFERENCE) by `make -C baseline`.
//
// Strategy: BlockStrategy<double, 128, 256, Architecture32>, the
// configuration of the reference's own GPU tests
// (tests/rpp/gpu/block/ops/gpu_block_test_helper.cuh:57-60), with the basis's
// degree table on the host as those tests pass it (the strategy maps it to
// the device on every launch).  Each wrapper takes raw device pointers, a
// batch stride and a degree range, and returns the reference's ErrorCode
// (0 = success).
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

#include <rpp/basis/tensor_basis.hpp>
#include <rpp/gpu/architecture.hpp>
#include <rpp/gpu/block/operations/basic/ft_adj_lmul.hpp>
#include <rpp/gpu/block/operations/basic/ft_adj_rmul.hpp>
#include <rpp/gpu/block/operations/basic/tensor_set_identity.hpp>
#include <rpp/gpu/block/operations/intermediate/ft_exp.hpp>
#include <rpp/gpu/block/operations/intermediate/ft_fmexp.hpp>
#include <rpp/gpu/strategies.hpp>
#include <rpp/views/dense_tensor_view.hpp>

namespace {

using Arch = rpp::gpu::arch::Architecture32;
using Strategy = rpp::gpu::strategies::BlockStrategy<double, 128, 256, Arch>;
using Index = Arch::Index;
using Degree = Arch::Degree;
using Basis = rpp::basis::TensorBasis<Arch>;
template <typename T>
using Ptr = Arch::Ptr<T>;

// Host degree table db[0..D+1] of one (width, depth), kept for the process.
struct HostBasis {
    Index db[40];
    Basis basis;
    HostBasis(Degree w, Degree d) : db{}, basis{w, d, db} {
        for (Degree n = 1; n <= d + 1; ++n) db[n] = 1 + static_cast<Index>(w) * db[n - 1];
    }
};

Basis basis_of(int width, int depth) {
    static HostBasis* cache[17][31] = {};
    if (!cache[width][depth]) cache[width][depth] = new HostBasis(width, depth);
    return cache[width][depth]->basis;
}

rpp::gpu::DeviceLaunchConfig config_of(void* stream) {
    rpp::gpu::DeviceLaunchConfig cfg;
    cfg.stream = static_cast<cudaStream_t>(stream);
    return cfg;
}

template <typename T>
auto batch(T* p, int64_t stride, int lo, int hi) {
    return rpp::make_tensor_batch(Ptr<T>(p), static_cast<Index>(stride), static_cast<Degree>(lo),
                                  static_cast<Degree>(hi));
}

template <typename E>
int code(const E& err) {
    return static_cast<bool>(err) ? 0 : static_cast<int>(err.code());
}

bool valid(int width, int depth) { return width >= 1 && width <= 16 && depth >= 1 && depth <= 30; }

}  // namespace

extern "C" {

int ref_block_tensor_set_identity(void* stream, int width, int depth, double* out, int64_t stride, int64_t n) {
    if (!valid(width, depth)) return -1;
    return code(rpp::ops::tensor_set_identity(Strategy{128}, config_of(stream), batch(out, stride, 0, depth),
                                              basis_of(width, depth), static_cast<Index>(n)));
}

int ref_block_ft_fmexp(void* stream, int width, int depth, double* out, int64_t out_stride, const double* mul,
                       int64_t mul_stride, const double* expo, int64_t exp_stride, int exp_lo, int exp_hi,
                       int64_t n) {
    if (!valid(width, depth)) return -1;
    return code(rpp::ops::ft_fmexp(Strategy{128}, config_of(stream), batch(out, out_stride, 0, depth),
                                   batch(mul, mul_stride, 0, depth), batch(expo, exp_stride, exp_lo, exp_hi),
                                   basis_of(width, depth), static_cast<Index>(n)));
}

int ref_block_ft_exp(void* stream, int width, int depth, double* out, int64_t out_stride, const double* arg,
                     int64_t arg_stride, int arg_lo, int arg_hi, int64_t n) {
    if (!valid(width, depth)) return -1;
    return code(rpp::ops::ft_exp(Strategy{128}, config_of(stream), batch(out, out_stride, 0, depth),
                                 batch(arg, arg_stride, arg_lo, arg_hi), basis_of(width, depth),
                                 static_cast<Index>(n)));
}

int ref_block_ft_adj_lmul(void* stream, int width, int depth, double* out, int64_t out_stride, const double* op,
                          int64_t op_stride, const double* arg, int64_t arg_stride, int64_t n) {
    if (!valid(width, depth)) return -1;
    return code(rpp::ops::ft_adj_lmul(Strategy{128}, config_of(stream), batch(out, out_stride, 0, depth),
                                      batch(op, op_stride, 0, depth), batch(arg, arg_stride, 0, depth),
                                      basis_of(width, depth), static_cast<Index>(n)));
}

int ref_block_ft_adj_rmul(void* stream, int width, int depth, double* out, int64_t out_stride, const double* op,
                          int64_t op_stride, const double* arg, int64_t arg_stride, int64_t n) {
    if (!valid(width, depth)) return -1;
    return code(rpp::ops::ft_adj_rmul(Strategy{128}, config_of(stream), batch(out, out_stride, 0, depth),
                                      batch(op, op_stride, 0, depth), batch(arg, arg_stride, 0, depth),
                                      basis_of(width, depth), static_cast<Index>(n)));
}

}  // extern "C"
