// sell.cuh -- one sparse matrix times one vector by a whole CTA, over the
// sliced copy of the matrix (CsrDevice: 32 rows per slice, rows by decreasing
// length, entry-major within a slice).  Used by the batched SpMM (sparse.cu)
// and by the fused Lie <-> tensor kernels (lie_fused.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ops.hpp"

namespace rpp_gb {

template <typename T>
__device__ __forceinline__ const T* sell_values(const CsrDevice& m);
template <>
__device__ __forceinline__ const double* sell_values<double>(const CsrDevice& m) {
    return m.ell_v64;
}
template <>
__device__ __forceinline__ const float* sell_values<float>(const CsrDevice& m) {
    return m.ell_v32;
}

// y[r] = alpha * sum_k val(r, k) x[col(r, k)] for every row r, entries in the
// row's CSR order (so the sum is rounded exactly as a row-by-row CSR product
// would round it); with a matrix that came from CSC, y[i] = alpha * 0 for
// rows <= i < zero_to as well (its product zeroes the whole output view).
// Slices go to warps in zig-zag order (round k: warp w takes slice
// k*warps + w for even k, k*warps + warps-1-w for odd k): slices are sorted
// longest first, so plain round-robin would give warp 0 the longest slice of
// every round (at W5 D5 the t2l matrix's busiest warp then has 1.65 times the
// mean work, 1.43 times in zig-zag order).  blockDim.x is a multiple of 32.
// Each y[r] is written once, by one thread.  Scale = false: alpha is 1 and
// is not multiplied in (chosen by the launchers at compile time).  Unroll:
// the entry loop unrolled 4x, so a lane issues the loads of several entries
// before their FMAs -- worth it for long rows (t2l at W5 D5, 12.7 entries per
// row: 0.128 -> 0.114 ms per 4096 vectors), slower for short ones (l2t, at
// most 5).  The sum keeps its single accumulator and entry order.
template <bool Scale, bool Unroll, typename T>
__device__ __forceinline__ void sell_rows(const CsrDevice& m, const T* __restrict__ x, T* y, int64_t zero_to,
                                          T alpha) {
    const T* vals = sell_values<T>(m);
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t slices = (m.rows + 31) / 32;
    for (int64_t round = 0; round * nw < slices; ++round) {
        const int64_t s = round * nw + ((round & 1) ? nw - 1 - w : w);
        const int64_t i = s * 32 + lane;
        if (s >= slices || i >= m.rows) continue;
        const int32_t r = __ldg(m.order + i), len = __ldg(m.row_len + i);
        const int32_t base = __ldg(m.slice_off + s) + static_cast<int32_t>(lane);
        T acc = T(0);
        if constexpr (Unroll) {
#pragma unroll 4
            for (int32_t k = 0; k < len; ++k) acc = fma(__ldg(vals + base + 32 * k), x[__ldg(m.ell_cols + base + 32 * k)], acc);
        } else {
            for (int32_t k = 0; k < len; ++k) acc = fma(__ldg(vals + base + 32 * k), x[__ldg(m.ell_cols + base + 32 * k)], acc);
        }
        y[r] = Scale ? alpha * acc : acc;
    }
    if (m.zero_rest)
        for (int64_t i = m.rows + threadIdx.x; i < zero_to; i += blockDim.x) y[i] = Scale ? alpha * T(0) : T(0);
}

}  // namespace rpp_gb
