// bulk_stage.cuh -- staging tensor levels into shared memory with the bulk
// copy engine (TMA, cp.async.bulk) instead of per-thread loads.
//
// One elected thread issues one cp.async.bulk per staged tensor, completing
// on an mbarrier in shared memory; the other threads meanwhile copy the
// ragged ends (a bulk copy moves 16-byte-aligned spans only) with plain
// loads.  A staged tensor keeps its element positions: element i of the
// source row lands at buffer + shift + i, where shift (< 16 / sizeof(T))
// gives the buffer the source row's alignment modulo 16 bytes, so every
// buffer holds dim + 16 / sizeof(T) elements.
//
// Waits are bounded: a wait that exceeds kBulkWaitLimit polls records
// kFaultBulkWait in the plan's fault word (Geometry::fault, read by
// rpp_gb_plan_fault) and returns, so a copy that never completes cannot hang
// the GPU; results of that launch are then invalid and the fault says so.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace rpp_gb {

constexpr uint32_t kFaultBulkWait = 1u;
constexpr uint32_t kBulkWaitLimit = 1u << 22;  // polls (each may suspend briefly)

// Elements of padding a staged buffer needs for the alignment shift.
template <typename T>
constexpr uint32_t stage_pad() {
    return 16u / sizeof(T);
}

// Elements of one staged buffer for a tensor of `dim` coefficients: the
// padding, rounded up so that consecutive buffers stay 16-byte aligned.
template <typename T>
__host__ __device__ constexpr uint32_t staged_elems(uint32_t dim) {
    return (dim + 2 * stage_pad<T>() - 1) / stage_pad<T>() * stage_pad<T>();
}

// Bytes at the start of dynamic shared memory holding the mbarrier.
constexpr uint32_t kBulkHeader = 16;

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t polls = 0; polls < limit; ++polls)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Generic-proxy accesses to shared memory before this point are ordered
// before later bulk-copy (async-proxy) writes to it.
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Stages levels of one or more tensors of the current batch element.  Usage
// (every thread of the CTA):
//     BulkStage<T> st(bar, phase);            // bar: 8 bytes of shared memory
//     T* P = st.add(buf_p, src_p, lo_p, hi_p, G);
//     T* A = st.add(buf_a, src_a, lo_a, hi_a, G);
//     st.commit(G.fault);                     // ends with a CTA barrier
// The mbarrier is initialised once per kernel (bulk_stage_init) and its phase
// flips on every commit.
template <typename T>
struct BulkStage {
    uint64_t* bar;
    uint32_t& phase;
    uint32_t bytes = 0;  // bulk bytes issued by thread 0 so far

    __device__ BulkStage(uint64_t* b, uint32_t& ph) : bar(b), phase(ph) {}

    // Buffer `buf` (dim + stage_pad<T>() elements) receives levels [lo, hi] of
    // the row at `src`; returns the pointer that plays the row's role.
    __device__ T* add(T* buf, const T* src, int lo, int hi, const Geometry& G) {
        if (lo > hi) return buf + static_cast<uint32_t>((reinterpret_cast<uintptr_t>(src) & 15u) / sizeof(T));
        return add_span(buf, src, G.db[lo], G.db[hi + 1]);
    }

    // Elements [b, e) of the row at `src` (buffer: e + stage_pad<T>() elements).
    __device__ T* add_span(T* buf, const T* src, uint32_t b, uint32_t e) {
        const uint32_t shift =
            static_cast<uint32_t>((reinterpret_cast<uintptr_t>(src) & 15u) / sizeof(T));
        T* dst = buf + shift;
        if (b >= e) return dst;
        // 16-byte aligned interior [ab, ae) of the source range
        constexpr uint32_t per16 = 16u / sizeof(T);
        const uint32_t lead = (per16 - ((shift + b) % per16)) % per16;
        uint32_t ab = b + lead;
        uint32_t ae = ab <= e ? e - ((e - ab) % per16) : ab;
        if (ab >= ae) ab = ae = e;  // too short for a bulk copy
        if (threadIdx.x == 0 && ae > ab) {
            const uint32_t nbytes = (ae - ab) * static_cast<uint32_t>(sizeof(T));
            bulk_copy_g2s(dst + ab, src + ab, nbytes, bar);
            bytes += nbytes;
        }
        for (uint32_t i = b + threadIdx.x; i < ab; i += blockDim.x) dst[i] = src[i];
        for (uint32_t i = ae + threadIdx.x; i < e; i += blockDim.x) dst[i] = src[i];
        return dst;
    }

    // Thread 0 declares the bulk bytes; everyone waits (bounded) for them and
    // for each other's edge copies.  Returns false on every thread when the
    // wait ran out: the fault is recorded, in-flight copies are waited for
    // once more (bounded) and the caller returns.
    __device__ bool commit(uint32_t* fault, uint32_t limit = kBulkWaitLimit) {
        if (threadIdx.x == 0) mbar_arrive_expect_tx(bar, bytes);
        bool done = mbar_wait_bounded(bar, phase, limit);
        if (!done) {
            if (fault) atomicOr(fault, kFaultBulkWait);
            done = mbar_wait_bounded(bar, phase, limit);
        }
        phase ^= 1u;
        return __syncthreads_and(done ? 1 : 0) != 0 && done;
    }
};

// Once per kernel, before the first staging: initialise the mbarrier (one
// arrival per phase: thread 0's arrive.expect_tx).
__device__ __forceinline__ void bulk_stage_init(uint64_t* bar) {
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
}

// Before re-staging into buffers the CTA has accessed with ordinary loads
// and stores: every thread orders its accesses before the async proxy's
// writes, then the barrier lets thread 0 issue the copies.
__device__ __forceinline__ void bulk_stage_reuse() {
    fence_proxy_async_shared();
    __syncthreads();
}

#endif  // __CUDACC__

}  // namespace rpp_gb
