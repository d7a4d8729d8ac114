// common.cuh -- shared device/host helpers of the sm_103a kernels.
//
// Basis geometry: a tensor of width W and depth D is stored degree-major with
// level n occupying [db[n], db[n+1]), db[n] = (W^n - 1)/(W - 1), level sizes
// pw[n] = W^n (include/rpp/basis/tensor_basis.hpp:40-130,
// include/rpp/basis/graded_basis.hpp:13-98).  Inside a level, index i of the
// word w_1..w_n is sum_j w_j W^(n-j): the split w = uv with |v| = k has
// u = i / W^k and v = i % W^k.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rpp_gb {

constexpr int kMaxDepth = 30;

// Division by a runtime-invariant 32-bit divisor via multiply-high, following
// Granlund & Montgomery, "Division by invariant integers using
// multiplication" (PLDI 1994), section 4: with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, q = (mulhi(m, n) + n) >> l for all
// n < 2^32.  The sum is formed in 64 bits so it cannot overflow.
struct FastDiv {
    uint32_t d;
    uint32_t m;
    uint32_t l;

    FastDiv() = default;
    __host__ explicit FastDiv(uint32_t divisor) : d(divisor) {
        l = 0;
        while ((uint64_t{1} << l) < divisor) ++l;
        m = static_cast<uint32_t>(((uint64_t{1} << 32) * ((uint64_t{1} << l) - divisor)) / divisor + 1);
    }
#if defined(__CUDACC__)
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        const uint32_t hi = __umulhi(m, n);
        return static_cast<uint32_t>((static_cast<uint64_t>(hi) + n) >> l);
    }
    __device__ __forceinline__ void divmod(uint32_t n, uint32_t& q, uint32_t& r) const {
        q = div(n);
        r = n - q * d;
    }
#endif
};

// Geometry of T^(D)(R^W), passed by value to every kernel (a few hundred bytes
// of constant-bank parameters).  Level sizes are kept below 2^31 so that the
// in-level index math is 32-bit.
struct Geometry {
    int32_t width;
    int32_t depth;
    uint32_t dim;
    uint32_t db[kMaxDepth + 2];
    uint32_t pw[kMaxDepth + 2];
    FastDiv divw;
    // The plan's fault word (device memory): kernels OR in a code when a
    // bounded wait runs out (rpp_gb_plan_fault reads and clears it).
    uint32_t* fault;
};

// One operand batch as seen by a kernel.
template <typename T>
struct TArg {
    T* p;
    int64_t stride;
    int32_t lo;
    int32_t hi;

    __host__ __device__ __forceinline__ bool has(int n) const { return lo <= n && n <= hi; }
    __host__ __device__ __forceinline__ T* at(int64_t b) const { return p + b * stride; }
};

#if defined(__CUDACC__)
__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
#endif

// Number of threads and blocks for a "one CTA per batch element" launch.
struct Launch {
    dim3 grid;
    dim3 block;
    size_t smem;
};

}  // namespace rpp_gb
