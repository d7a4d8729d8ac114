// launch_util.cuh -- launch-shape helpers shared by the kernel files.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "ops.hpp"

namespace rpp_gb {

constexpr int kMaxDevices = 64;

// Raise a kernel's dynamic shared-memory ceiling to the device's opt-in maximum
// once per (kernel, device).  The kernel is a template argument so that every
// kernel gets its own flag array, even kernels of identical signature.
template <auto kernel>
inline cudaError_t allow_large_smem(const DeviceInfo& dev) {
    static std::atomic<bool> done[kMaxDevices];
    if (dev.device < 0 || dev.device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (done[dev.device].load(std::memory_order_acquire)) return cudaSuccess;
    // static + dynamic shared memory must fit the opt-in limit
    cudaFuncAttributes attr{};
    cudaError_t err = cudaFuncGetAttributes(&attr, kernel);
    if (err != cudaSuccess) return err;
    const int dynamic_max = dev.max_smem_optin - static_cast<int>(attr.sharedSizeBytes);
    err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dynamic_max);
    if (err == cudaSuccess) done[dev.device].store(true, std::memory_order_release);
    return err;
}

// Grid for a "one CTA per batch element, grid-stride over the batch" kernel:
// as many CTAs as fit on the device at once, capped by the batch.
template <typename Kernel>
inline cudaError_t batch_grid(Kernel kernel, const DeviceInfo& dev, int threads, size_t smem,
                              int64_t batch, dim3& grid) {
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int64_t cap = static_cast<int64_t>(per_sm) * dev.sm_count;
    grid = dim3(static_cast<unsigned>(std::max<int64_t>(1, std::min(batch, cap))));
    return cudaSuccess;
}

// Threads per CTA for a tensor whose largest level has `widest` coefficients.
inline int threads_for(uint32_t widest, int cap = 256) {
    int t = 32;
    while (t < cap && static_cast<uint32_t>(t) < widest) t *= 2;
    return t;
}

}  // namespace rpp_gb
