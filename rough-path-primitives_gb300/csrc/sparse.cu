// sparse.cu -- batched sparse matrix x dense vectors (SpMM) for
// tensor_to_lie / lie_to_tensor / sparse_matrix_vector_product.
//
// The reference launches one CTA per vector and, for CSC, one thread per
// non-zero with a binary search for its column and a block-scope atomic add
// into global memory (include/rpp/gpu/block/operations/linalg/
// sparse_matrix_vector.hpp:150-185).  Here the matrix is CSR (CSC inputs are
// transposed once when the handle is created), each CTA stages one argument
// vector in shared memory and each thread owns output rows: no atomics, a
// deterministic summation order, coalesced writes.
#include "bulk_stage.cuh"
#include "common.cuh"
#include "launch_util.cuh"
#include "ops.hpp"

namespace rpp_gb {
namespace {

template <typename T>
__device__ __forceinline__ const T* csr_values(const CsrDevice& m);
template <>
__device__ __forceinline__ const double* csr_values<double>(const CsrDevice& m) {
    return m.values64;
}
template <>
__device__ __forceinline__ const float* csr_values<float>(const CsrDevice& m) {
    return m.values32;
}

template <typename T>
__global__ void __launch_bounds__(256) k_spmm(CsrDevice m, T* out, int64_t out_stride, int64_t out_size,
                                              const T* arg, int64_t arg_stride, int64_t arg_size,
                                              int64_t batch, T alpha, int staged) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* s_arg = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    uint32_t phase = 0;
    if (staged) bulk_stage_init(bar);
    const T* vals = csr_values<T>(m);
    const int64_t rows = m.rows;
    const int64_t write_end = m.zero_rest ? out_size : rows;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const T* x = arg + b * arg_stride;
        T* y = out + b * out_stride;
        if (staged) {
            BulkStage<T> st(bar, phase);
            x = st.add_span(s_arg, x, 0, static_cast<uint32_t>(arg_size));
            if (!st.commit(m.fault)) return;
        }
        for (int64_t r = threadIdx.x; r < write_end; r += blockDim.x) {
            T acc = T(0);
            if (r < rows) {
                const int32_t e0 = __ldg(m.offsets + r), e1 = __ldg(m.offsets + r + 1);
                for (int32_t e = e0; e < e1; ++e) acc = fma(__ldg(vals + e), x[__ldg(m.cols + e)], acc);
            }
            y[r] = alpha * acc;
        }
        if (staged) bulk_stage_reuse();
    }
}

}  // namespace

template <typename T>
cudaError_t launch_spmm(const CsrDevice& m, const DeviceInfo& dev, cudaStream_t s, T* out,
                        int64_t out_stride, int64_t out_size, const T* arg, int64_t arg_stride,
                        int64_t arg_size, int64_t batch, double alpha) {
    if (batch <= 0) return cudaSuccess;
    constexpr auto kernel = k_spmm<T>;
    cudaError_t err = allow_large_smem<kernel>(dev);
    if (err != cudaSuccess) return err;
    const size_t need = kBulkHeader + static_cast<size_t>(staged_elems<T>(static_cast<uint32_t>(arg_size))) * sizeof(T);
    const int staged = arg_size < (int64_t{1} << 31) && need <= 96 * 1024;
    const size_t smem = staged ? need : 0;
    const int threads = 256;
    dim3 grid;
    if ((err = batch_grid(kernel, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
    kernel<<<grid, threads, smem, s>>>(m, out, out_stride, out_size, arg, arg_stride, arg_size, batch,
                                       static_cast<T>(alpha), staged);
    return cudaGetLastError();
}

template cudaError_t launch_spmm<float>(const CsrDevice&, const DeviceInfo&, cudaStream_t, float*, int64_t,
                                        int64_t, const float*, int64_t, int64_t, int64_t, double);
template cudaError_t launch_spmm<double>(const CsrDevice&, const DeviceInfo&, cudaStream_t, double*,
                                         int64_t, int64_t, const double*, int64_t, int64_t, int64_t,
                                         double);

}  // namespace rpp_gb
