// sparse.cu -- batched sparse matrix x dense vectors (SpMM) for
// tensor_to_lie / lie_to_tensor / sparse_matrix_vector_product.
//
// The reference launches one CTA per vector and, for CSC, one thread per
// non-zero with a binary search for its column and a block-scope atomic add
// into global memory (include/rpp/gpu/block/operations/linalg/
// sparse_matrix_vector.hpp:150-185).  Here the matrix is converted once, when
// the handle is created, to CSR (CSC inputs transposed) and to a sliced copy
// of 32 rows per slice (sell.cuh); each CTA stages one argument vector in
// shared memory and each thread owns output rows: no atomics and a
// deterministic summation order.
#include <type_traits>

#include "bulk_stage.cuh"
#include "common.cuh"
#include "launch_util.cuh"
#include "ops.hpp"
#include "sell.cuh"

namespace rpp_gb {
namespace {

template <typename T, bool Scale, bool Unroll>
__global__ void __launch_bounds__(256) k_spmm(CsrDevice m, T* out, int64_t out_stride, int64_t out_size,
                                              const T* arg, int64_t arg_stride, int64_t arg_size,
                                              int64_t batch, T alpha, int staged) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* s_arg = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    uint32_t phase = 0;
    if (staged) bulk_stage_init(bar);
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const T* x = arg + b * arg_stride;
        T* y = out + b * out_stride;
        if (staged) {
            BulkStage<T> st(bar, phase);
            x = st.add_span(s_arg, x, 0, static_cast<uint32_t>(arg_size));
            if (!st.commit(m.fault)) return;
        }
        sell_rows<Scale, Unroll>(m, x, y, out_size, alpha);
        if (staged) bulk_stage_reuse();
    }
}

}  // namespace

template <typename T>
cudaError_t launch_spmm(const CsrDevice& m, const DeviceInfo& dev, cudaStream_t s, T* out,
                        int64_t out_stride, int64_t out_size, const T* arg, int64_t arg_stride,
                        int64_t arg_size, int64_t batch, double alpha) {
    if (batch <= 0) return cudaSuccess;
    const size_t need = kBulkHeader + static_cast<size_t>(staged_elems<T>(static_cast<uint32_t>(arg_size))) * sizeof(T);
    const int staged = arg_size < (int64_t{1} << 31) && need <= 96 * 1024;
    const size_t smem = staged ? need : 0;
    const int threads = 256;
    auto run = [&](auto kernel) {
        constexpr auto k = decltype(kernel)::value;
        cudaError_t err = allow_large_smem<k>(dev);
        if (err != cudaSuccess) return err;
        dim3 grid;
        if ((err = batch_grid(k, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
        k<<<grid, threads, smem, s>>>(m, out, out_stride, out_size, arg, arg_stride, arg_size, batch,
                                      static_cast<T>(alpha), staged);
        return cudaGetLastError();
    };
    const bool one = static_cast<T>(alpha) == T(1), longrows = m.nnz >= 8 * m.rows;  // (sell.cuh)
    if (one && longrows) return run(std::integral_constant<decltype(&k_spmm<T, false, true>), &k_spmm<T, false, true>>{});
    if (one) return run(std::integral_constant<decltype(&k_spmm<T, false, false>), &k_spmm<T, false, false>>{});
    if (longrows) return run(std::integral_constant<decltype(&k_spmm<T, true, true>), &k_spmm<T, true, true>>{});
    return run(std::integral_constant<decltype(&k_spmm<T, true, false>), &k_spmm<T, true, false>>{});
}

template cudaError_t launch_spmm<float>(const CsrDevice&, const DeviceInfo&, cudaStream_t, float*, int64_t,
                                        int64_t, const float*, int64_t, int64_t, int64_t, double);
template cudaError_t launch_spmm<double>(const CsrDevice&, const DeviceInfo&, cudaStream_t, double*,
                                         int64_t, int64_t, const double*, int64_t, int64_t, int64_t,
                                         double);

}  // namespace rpp_gb
