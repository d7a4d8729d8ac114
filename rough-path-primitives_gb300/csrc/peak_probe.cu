// peak_probe.cu -- FMA-throughput probe used as the roofline denominator of
// the FMA-bound kernels (the device's FP64 rate is not a published constant
// one can trust for a given clock, so the benchmark measures it in-run), and
// the self-test of the bounded mbarrier wait used by the staging helper.
//
// Every thread runs 8 independent FMA chains; the grid is 8 CTAs of 256
// threads per SM, which saturates the FP64 pipes of all four sub-partitions.
#include <cuda_runtime.h>

#include "../../include/rpp_gb300.h"
#include "bulk_stage.cuh"
#include "ops.hpp"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, int iters, T a, T b) {
    T acc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = static_cast<T>(threadIdx.x + c) * static_cast<T>(1e-3);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] = fma(acc[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
cudaError_t probe(int device, int iters, double* tflops) {
    int sms = 0;
    cudaError_t err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (err != cudaSuccess) return err;
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    if ((err = cudaMalloc(&out, sizeof(T) * blocks * threads)) != cudaSuccess) return err;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int w = 0; w < 2; ++w) k_fma_probe<T><<<blocks, threads>>>(out, iters, T(0.999), T(1e-4));
    cudaEventRecord(e0);
    const int reps = 3;
    for (int r = 0; r < reps; ++r) k_fma_probe<T><<<blocks, threads>>>(out, iters, T(0.999), T(1e-4));
    cudaEventRecord(e1);
    err = cudaEventSynchronize(e1);
    float ms = 0;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err == cudaSuccess) err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err == cudaSuccess && ms > 0)
        *tflops = 2.0 * reps * double(blocks) * threads * double(iters) * 8 / (ms * 1e-3) / 1e12;
    return err;
}

}  // namespace

extern "C" int rpp_gb_fma_peak(int32_t dtype, int32_t device, double* tflops) {
    if (!tflops || (dtype != RPP_GB_F32 && dtype != RPP_GB_F64)) return RPP_GB_INVALID_ARGUMENT;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return RPP_GB_INVALID_ARGUMENT;
    cudaError_t err = dtype == RPP_GB_F64 ? probe<double>(device, 2000, tflops) : probe<float>(device, 20000, tflops);
    cudaSetDevice(prev);
    return err == cudaSuccess ? RPP_GB_SUCCESS : RPP_GB_INTERNAL;
}

namespace rpp_gb {
namespace {

// Declares 16 bytes of transaction on an mbarrier and issues no copy, so the
// phase never completes; the bounded commit must expire (limit 4096 polls),
// record the fault and return on every thread.
__global__ void k_expired_wait(uint32_t* fault) {
    __shared__ __align__(8) uint64_t bar;
    bulk_stage_init(&bar);
    uint32_t phase = 0;
    BulkStage<double> st(&bar, phase);
    st.bytes = 16;
    st.commit(fault, 4096);
}

}  // namespace

cudaError_t launch_expired_wait(const Geometry& g, cudaStream_t s) {
    k_expired_wait<<<1, 32, 0, s>>>(g.fault);
    return cudaGetLastError();
}

}  // namespace rpp_gb

