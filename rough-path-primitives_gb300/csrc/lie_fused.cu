// lie_fused.cu -- the steps either side of the signature, fused per tensor.
//
// Log-signature epilogue: out = alpha * T2L * log(x), where log is
// rpp::ops::ft_log (include/rpp/operations/intermediate/ft_log.hpp:87-114)
// on the degree range [lo, hi] and T2L is the tensor_to_lie matrix
// (include/rpp/operations/basic/tensor_to_lie.hpp:65-103, built by
// include/rpp/sparse/t2l_matrix.hpp:57-142) applied to that view with the
// begin-relative indexing of the CPU strategy's SpMV.  The reference composes
// two launches with the full log tensor in between; here the log stays in
// shared memory and only the Lie coefficients are written.
//
// Lie-increment step: X = alpha * L2T * lambda written to degrees [lo, hi] of a
// zero tensor (rpp::ops::lie_to_tensor, lie_to_tensor.hpp:70-108, matrix from
// include/rpp/sparse/l2t_matrix.hpp:58-114), then out = exp(X)
// (ft_exp.hpp) or out = M (x) exp(X) (ft_fmexp.hpp:91-121): one log-ODE step of
// a path given by Lie increments.  X never leaves shared memory.
//
// Both kernels hold one tensor of the batch per CTA (grid-stride) and need
// two work tensors in shared memory (the multiplier of the Lie step is read
// from global memory); the host composes the unfused kernels for states that
// do not fit.
#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>

#include "bulk_stage.cuh"
#include "ft_device.cuh"
#include "launch_util.cuh"
#include "ops.hpp"
#include "sell.cuh"

namespace rpp_gb {
namespace {

using namespace ftdev;

template <typename T, bool Scale>
__global__ void __launch_bounds__(256) k_log_to_lie(Geometry G, CsrDevice m, TArg<T> x, int lo, int hi, T* out,
                                                   int64_t out_stride, int64_t out_size, int64_t batch, T alpha) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* s_x = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    T* s_log = s_x + staged_elems<T>(G.dim);
    uint32_t phase = 0;
    bulk_stage_init(bar);
    const Opnd<T> none{nullptr, 1, 0};
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        Opnd<T> X{x.at(b), imax(1, x.lo), imin(x.hi, G.depth)};
        BulkStage<T> st(bar, phase);
        X.p = st.add(s_x, X.p, X.lo, X.hi, G);
        if (!st.commit(G.fault)) return;
        intermediate_one(G, IntermediateKind::Log, s_log, lo, hi, X, none);
        __syncthreads();
        sell_rows<Scale, true>(m, s_log + G.db[lo], out + b * out_stride, out_size, alpha);  // t2l: long rows
        bulk_stage_reuse();
    }
}

template <typename T, bool Scale>
__global__ void __launch_bounds__(256) k_lie_exp(Geometry G, CsrDevice m, const T* lie, int64_t lie_stride, int lo,
                                                int hi, TArg<T> out, TArg<T> mult, int64_t batch, T alpha) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    const uint32_t pd = staged_elems<T>(G.dim);
    T* s_x = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    T* s_o = s_x + pd;  // also holds the Lie vector until X is formed
    uint32_t phase = 0;
    bulk_stage_init(bar);
    const int ohi = imin(out.hi, G.depth);
    const bool fm = mult.p != nullptr;
    const uint32_t view = G.db[hi + 1] - G.db[lo];
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        BulkStage<T> st(bar, phase);
        const T* l = st.add_span(s_o, lie + b * lie_stride, 0, static_cast<uint32_t>(m.cols_dim));
        // the multiplier stays in global memory (each coefficient is read once
        // per Horner round, from L1/L2), so the CTA holds two tensors, not three
        Opnd<T> M{nullptr, 1, 0};
        if (fm) M = {mult.at(b), mult.lo, imin(mult.hi, G.depth)};
        for (uint32_t i = threadIdx.x; i < G.dim; i += blockDim.x) s_x[i] = T(0);
        if (!st.commit(G.fault)) return;
        sell_rows<Scale, false>(m, l, s_x + G.db[lo], static_cast<int64_t>(view), alpha);  // l2t: short rows
        __syncthreads();
        const Opnd<T> X{s_x, imax(1, lo), hi};
        intermediate_one(G, fm ? IntermediateKind::FMExp : IntermediateKind::Exp, s_o, out.lo, ohi, X, M);
        __syncthreads();
        T* o = out.at(b);
        if (out.lo <= ohi)
            for (uint32_t i = G.db[out.lo] + threadIdx.x; i < G.db[ohi + 1]; i += blockDim.x) o[i] = s_o[i];
        bulk_stage_reuse();
    }
}

}  // namespace

// Staged buffers carry the bulk copy's alignment padding (bulk_stage.cuh).
static size_t staged_bytes(const Geometry& g, size_t elem) {
    const size_t per16 = 16 / elem;
    return (g.dim + 2 * per16 - 1) / per16 * per16 * elem;
}
size_t log_to_lie_smem(const Geometry& g, size_t elem) { return kBulkHeader + 2 * staged_bytes(g, elem); }
size_t lie_exp_smem(const Geometry& g, size_t elem, bool fm) {
    (void)fm;  // the multiplier is read from global memory
    return kBulkHeader + 2 * staged_bytes(g, elem);
}

template <typename T>
cudaError_t launch_log_to_lie(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const CsrDevice& m,
                              TArg<T> x, int lo, int hi, T* out, int64_t out_stride, int64_t out_size, int64_t batch,
                              double alpha) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = log_to_lie_smem(g, sizeof(T));
    if (smem > static_cast<size_t>(dev.max_smem_optin)) return cudaErrorInvalidConfiguration;
    const int threads = threads_for(g.pw[g.depth]);
    auto run = [&](auto kernel) {
        constexpr auto k = decltype(kernel)::value;
        cudaError_t err = allow_large_smem<k>(dev);
        if (err != cudaSuccess) return err;
        dim3 grid;
        if ((err = batch_grid(k, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
        k<<<grid, threads, smem, s>>>(g, m, x, lo, hi, out, out_stride, out_size, batch, static_cast<T>(alpha));
        return cudaGetLastError();
    };
    if (static_cast<T>(alpha) == T(1))
        return run(std::integral_constant<decltype(&k_log_to_lie<T, false>), &k_log_to_lie<T, false>>{});
    return run(std::integral_constant<decltype(&k_log_to_lie<T, true>), &k_log_to_lie<T, true>>{});
}

template <typename T>
cudaError_t launch_lie_exp(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const CsrDevice& m,
                           const T* lie, int64_t lie_stride, int lo, int hi, TArg<T> out, TArg<T> mult,
                           int64_t batch, double alpha) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = lie_exp_smem(g, sizeof(T), mult.p != nullptr);
    if (smem > static_cast<size_t>(dev.max_smem_optin) || m.cols_dim > static_cast<int64_t>(g.dim))
        return cudaErrorInvalidConfiguration;
    const int threads = threads_for(g.pw[g.depth]);
    auto run = [&](auto kernel) {
        constexpr auto k = decltype(kernel)::value;
        cudaError_t err = allow_large_smem<k>(dev);
        if (err != cudaSuccess) return err;
        dim3 grid;
        if ((err = batch_grid(k, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
        k<<<grid, threads, smem, s>>>(g, m, lie, lie_stride, lo, hi, out, mult, batch, static_cast<T>(alpha));
        return cudaGetLastError();
    };
    if (static_cast<T>(alpha) == T(1))
        return run(std::integral_constant<decltype(&k_lie_exp<T, false>), &k_lie_exp<T, false>>{});
    return run(std::integral_constant<decltype(&k_lie_exp<T, true>), &k_lie_exp<T, true>>{});
}

#define RPP_GB_INSTANTIATE_LIE_FUSED(T)                                                                           \
    template cudaError_t launch_log_to_lie<T>(const Geometry&, const DeviceInfo&, cudaStream_t, const CsrDevice&, \
                                              TArg<T>, int, int, T*, int64_t, int64_t, int64_t, double);          \
    template cudaError_t launch_lie_exp<T>(const Geometry&, const DeviceInfo&, cudaStream_t, const CsrDevice&,    \
                                           const T*, int64_t, int, int, TArg<T>, TArg<T>, int64_t, double);

RPP_GB_INSTANTIATE_LIE_FUSED(float)
RPP_GB_INSTANTIATE_LIE_FUSED(double)

}  // namespace rpp_gb
