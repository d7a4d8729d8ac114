// capi.cpp -- the C ABI of include/rpp_gb300.h: plans, matrix handles,
// argument validation, error mapping and dispatch to the kernel launchers.
//
// Error convention: every entry point returns an rpp::ErrorCode value
// (include/rpp/support/error.hpp:28-39) and records a message readable with
// rpp_gb_last_error_string() on the same host thread.  CUDA runtime errors
// are classified like the reference's map_cuda_error
// (include/rpp/gpu/device.hpp:27-140).
#include <cuda_runtime.h>

#include <algorithm>
#include <utility>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <type_traits>
#include <string>
#include <vector>

#include "../../include/rpp_gb300.h"
#include "lie_tables.hpp"
#include "ops.hpp"

struct rpp_gb_plan {
    rpp_gb::Geometry geometry;
    rpp_gb::DeviceInfo device;
};

struct rpp_gb_matrix {
    rpp_gb::CsrDevice csr;
    int32_t device;
    void* allocation;  // one device block holding offsets, cols and both value arrays
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int ok() {
    g_last_error.clear();
    return RPP_GB_SUCCESS;
}

int map_cuda(cudaError_t err) {
    switch (err) {
        case cudaSuccess:
            return RPP_GB_SUCCESS;
        case cudaErrorInvalidValue:
        case cudaErrorInvalidDevice:
        case cudaErrorInvalidSymbol:
        case cudaErrorInvalidPitchValue:
        case cudaErrorInvalidResourceHandle:
        case cudaErrorInvalidConfiguration:
        case cudaErrorInvalidClusterSize:
        case cudaErrorInvalidKernelImage:
        case cudaErrorInvalidPtx:
        case cudaErrorInvalidSource:
        case cudaErrorInvalidDevicePointer:
            return RPP_GB_INVALID_ARGUMENT;
        case cudaErrorMemoryAllocation:
        case cudaErrorLaunchOutOfResources:
        case cudaErrorOperatingSystem:
        case cudaErrorInitializationError:
        case cudaErrorInsufficientDriver:
        case cudaErrorNoDevice:
        case cudaErrorDevicesUnavailable:
            return RPP_GB_OUT_OF_RESOURCES;
        case cudaErrorLaunchTimeout:
            return RPP_GB_TIMEOUT;
        case cudaErrorNotReady:
            return RPP_GB_CANCELLED;
        case cudaErrorNotSupported:
        case cudaErrorUnsupportedLimit:
        case cudaErrorUnsupportedPtxVersion:
        case cudaErrorJitCompilerNotFound:
        case cudaErrorCallRequiresNewerDriver:
        case cudaErrorStreamCaptureUnsupported:
        case cudaErrorNoKernelImageForDevice:
            return RPP_GB_NOT_IMPLEMENTED;
        case cudaErrorLaunchFailure:
        case cudaErrorAssert:
        case cudaErrorIllegalState:
        case cudaErrorStreamCaptureInvalidated:
        case cudaErrorStreamCaptureMerge:
        case cudaErrorStreamCaptureUnmatched:
        case cudaErrorStreamCaptureUnjoined:
        case cudaErrorStreamCaptureIsolation:
        case cudaErrorStreamCaptureImplicit:
        case cudaErrorCapturedEvent:
        case cudaErrorStreamCaptureWrongThread:
        case cudaErrorIllegalAddress:
        case cudaErrorIllegalInstruction:
        case cudaErrorMisalignedAddress:
        case cudaErrorHardwareStackError:
            return RPP_GB_CONTRACT_VIOLATION;
        case cudaErrorECCUncorrectable:
        case cudaErrorSharedObjectSymbolNotFound:
        case cudaErrorSharedObjectInitFailed:
        case cudaErrorStartupFailure:
        case cudaErrorCudartUnloading:
        case cudaErrorSystemNotReady:
        case cudaErrorSystemDriverMismatch:
        case cudaErrorUnknown:
            return RPP_GB_INTERNAL;
        default:
            return RPP_GB_UNKNOWN;
    }
}

int cuda_status(cudaError_t err, const char* where) {
    if (err == cudaSuccess) return ok();
    return fail(map_cuda(err), std::string(where) + ": " + cudaGetErrorString(err));
}

// Make the plan's device current for the duration of a call.
class DeviceGuard {
public:
    explicit DeviceGuard(int device) {
        cudaGetDevice(&prev_);
        if (prev_ != device) {
            err_ = cudaSetDevice(device);
            switched_ = err_ == cudaSuccess;
        }
    }
    ~DeviceGuard() {
        if (switched_) cudaSetDevice(prev_);
    }
    cudaError_t error() const { return err_; }

private:
    int prev_ = 0;
    bool switched_ = false;
    cudaError_t err_ = cudaSuccess;
};

bool valid_dtype(int32_t dtype) { return dtype == RPP_GB_F32 || dtype == RPP_GB_F64; }

// Normalise a view's degree range to [lo, min(hi, depth)] (empty when lo > hi).
// Outputs (is_output) must not overlap between batch elements; inputs may
// use any non-negative stride, including 0 to broadcast one tensor.
template <typename T>
bool to_targ(const rpp_gb_tensor_arg* a, const rpp_gb::Geometry& g, bool required, int64_t batch,
             rpp_gb::TArg<T>& out, const char* name, bool is_output = false) {
    out = rpp_gb::TArg<T>{nullptr, 0, 1, 0};
    if (!a) {
        if (required) {
            fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + " is NULL");
            return false;
        }
        return true;
    }
    if (a->min_degree < 0) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + ": negative min_degree");
        return false;
    }
    if (a->stride < 0) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + ": negative batch stride");
        return false;
    }
    const int32_t hi = std::min<int32_t>(a->max_degree, g.depth);
    const bool empty = a->min_degree > hi;
    if (!a->data && !empty && batch > 0) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + ": NULL data for a non-empty view");
        return false;
    }
    if (is_output && !empty && a->stride < static_cast<int64_t>(g.db[hi + 1]) && batch > 1) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + ": stride shorter than the view");
        return false;
    }
    out.p = static_cast<T*>(a->data);
    out.stride = a->stride;
    out.lo = empty ? 1 : a->min_degree;
    out.hi = empty ? 0 : hi;
    return true;
}

template <typename F>
int with_plan(const rpp_gb_plan* plan, int32_t dtype, int64_t batch, F&& body) {
    if (!plan) return fail(RPP_GB_INVALID_ARGUMENT, "plan is NULL");
    if (!valid_dtype(dtype)) return fail(RPP_GB_INVALID_ARGUMENT, "unknown dtype");
    if (batch < 0) return fail(RPP_GB_INVALID_ARGUMENT, "negative batch size");
    if (batch == 0) return ok();
    DeviceGuard guard(plan->device.device);
    if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");
    return body();
}

template <typename T>
int run_product(const rpp_gb_plan* plan, cudaStream_t s, rpp_gb::ProductKind kind, const rpp_gb_tensor_arg* out,
                const rpp_gb_tensor_arg* x, const rpp_gb_tensor_arg* y, const rpp_gb_tensor_arg* z,
                int64_t batch, double alpha, double beta, bool need_x) {
    rpp_gb::TArg<T> o, a, b, c;
    const auto& g = plan->geometry;
    if (!to_targ(out, g, true, batch, o, "out", true) || !to_targ(x, g, need_x, batch, a, "a") ||
        !to_targ(y, g, true, batch, b, "b") || !to_targ(z, g, kind != rpp_gb::ProductKind::InplaceMul, batch, c, "c"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    return cuda_status(rpp_gb::launch_product<T>(g, plan->device, s, kind, o, a, b, c, batch, alpha, beta),
                       "product kernel");
}

int run_product_any(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, rpp_gb::ProductKind kind,
                    const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* x, const rpp_gb_tensor_arg* y,
                    const rpp_gb_tensor_arg* z, int64_t batch, double alpha, double beta, bool need_x) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_product<double>(plan, s, kind, out, x, y, z, batch, alpha, beta, need_x)
                                   : run_product<float>(plan, s, kind, out, x, y, z, batch, alpha, beta, need_x);
    });
}

template <typename T>
int run_intermediate(const rpp_gb_plan* plan, cudaStream_t s, rpp_gb::IntermediateKind kind,
                     const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* x, const rpp_gb_tensor_arg* m,
                     int64_t batch) {
    rpp_gb::TArg<T> o, a, b;
    const auto& g = plan->geometry;
    if (!to_targ(out, g, true, batch, o, "out", true) || !to_targ(x, g, true, batch, a, "arg") ||
        !to_targ(m, g, kind == rpp_gb::IntermediateKind::FMExp, batch, b, "multiplier"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    if (kind == rpp_gb::IntermediateKind::FMExp && out->data == m->data && batch > 0)
        return fail(RPP_GB_INVALID_ARGUMENT, "ft_fmexp: out must not alias multiplier");
    return cuda_status(rpp_gb::launch_intermediate<T>(g, plan->device, s, kind, o, a, b, batch),
                       "intermediate kernel");
}

int run_intermediate_any(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                         rpp_gb::IntermediateKind kind, const rpp_gb_tensor_arg* out,
                         const rpp_gb_tensor_arg* x, const rpp_gb_tensor_arg* m, int64_t batch) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_intermediate<double>(plan, s, kind, out, x, m, batch)
                                   : run_intermediate<float>(plan, s, kind, out, x, m, batch);
    });
}

template <typename T>
int run_adjoint(const rpp_gb_plan* plan, cudaStream_t s, bool left, const rpp_gb_tensor_arg* out,
                const rpp_gb_tensor_arg* op, const rpp_gb_tensor_arg* arg, int64_t batch) {
    rpp_gb::TArg<T> o, p, a;
    const auto& g = plan->geometry;
    if (!to_targ(out, g, true, batch, o, "out", true) || !to_targ(op, g, true, batch, p, "op") ||
        !to_targ(arg, g, true, batch, a, "arg"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    return cuda_status(rpp_gb::launch_adjoint<T>(g, plan->device, s, left, o, p, a, batch), "adjoint kernel");
}

template <typename T>
int run_helper(const rpp_gb_plan* plan, cudaStream_t s, rpp_gb::HelperKind kind, const rpp_gb_tensor_arg* out,
               const rpp_gb_tensor_arg* arg, int64_t batch, double value) {
    rpp_gb::TArg<T> o, a;
    const auto& g = plan->geometry;
    if (!to_targ(out, g, true, batch, o, "out", true) ||
        !to_targ(arg, g, kind == rpp_gb::HelperKind::Assign, batch, a, "arg"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    return cuda_status(rpp_gb::launch_helper<T>(g, plan->device, s, kind, o, a, batch, value), "helper kernel");
}

int run_helper_any(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, rpp_gb::HelperKind kind,
                   const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* arg, int64_t batch, double value) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_helper<double>(plan, s, kind, out, arg, batch, value)
                                   : run_helper<float>(plan, s, kind, out, arg, batch, value);
    });
}

// Schedules chosen by rpp_gb_signature_tune, keyed by the call's shape:
// (device, width, depth, dtype, mode, ragged).  Read by every signature call.
struct ScheduleKey {
    int device, width, depth, dtype, mode, ragged;
    bool operator<(const ScheduleKey& o) const {
        return std::tie(device, width, depth, dtype, mode, ragged) <
               std::tie(o.device, o.width, o.depth, o.dtype, o.mode, o.ragged);
    }
};
std::mutex g_schedule_lock;
std::map<ScheduleKey, int> g_schedules;

ScheduleKey schedule_key(const rpp_gb_plan* plan, int32_t dtype, bool forward, const void* sig, const void* seed,
                         const int64_t* offsets) {
    const int mode = (forward ? 1 : 0) | (seed ? 2 : 0) | (sig ? 4 : 0);
    return ScheduleKey{plan->device.device, plan->geometry.width, plan->geometry.depth, dtype, mode,
                       offsets != nullptr ? 1 : 0};
}

int scheduled_threads(const ScheduleKey& key) {
    std::lock_guard<std::mutex> guard(g_schedule_lock);
    auto it = g_schedules.find(key);
    return it == g_schedules.end() ? 0 : it->second;
}

template <typename T>
int check_signature_args(const rpp_gb_plan* plan, const void* incr, const int64_t* offsets, int64_t length,
                         const void* sig, int64_t sig_stride, const void* seed, int64_t seed_stride,
                         const void* grad, bool forward) {
    const auto& g = plan->geometry;
    if (!offsets && length < 0) return fail(RPP_GB_INVALID_ARGUMENT, "negative path length");
    if (!incr && (offsets || length > 0)) return fail(RPP_GB_INVALID_ARGUMENT, "increments are NULL");
    if (sig && sig_stride < static_cast<int64_t>(g.dim))
        return fail(RPP_GB_INVALID_ARGUMENT, "signature stride shorter than the tensor dimension");
    if (seed && seed_stride < static_cast<int64_t>(g.dim))
        return fail(RPP_GB_INVALID_ARGUMENT, "seed stride shorter than the tensor dimension");
    if ((seed == nullptr) != (grad == nullptr))
        return fail(RPP_GB_INVALID_ARGUMENT, "seed and grad must be given together");
    if (!forward && (!sig || !seed))
        return fail(RPP_GB_INVALID_ARGUMENT, "backward needs the final signatures and the seeds");
    if (forward && !sig && !grad) return fail(RPP_GB_INVALID_ARGUMENT, "nothing to compute");
    if (static_cast<int64_t>(g.depth) * g.width > 256)
        return fail(RPP_GB_NOT_IMPLEMENTED, "signature kernels need depth*width <= 256");
    return RPP_GB_SUCCESS;
}

template <typename T>
int run_signature(const rpp_gb_plan* plan, cudaStream_t s, int32_t dtype, const void* incr, const int64_t* offsets,
                  int64_t length, int64_t batch, void* sig, int64_t sig_stride, const void* seed,
                  int64_t seed_stride, void* grad, bool forward, int threads = -1) {
    if (int rc = check_signature_args<T>(plan, incr, offsets, length, sig, sig_stride, seed, seed_stride, grad,
                                         forward))
        return rc;
    if (threads < 0) threads = scheduled_threads(schedule_key(plan, dtype, forward, sig, seed, offsets));
    rpp_gb::PathBatch paths{offsets, length, batch};
    return cuda_status(rpp_gb::launch_signature<T>(plan->geometry, plan->device, s, static_cast<const T*>(incr),
                                                   paths, static_cast<T*>(sig), sig_stride,
                                                   static_cast<const T*>(seed), seed_stride, static_cast<T*>(grad),
                                                   forward, threads),
                       "signature kernel");
}

// Autotuner: time each candidate schedule (CTA size, optionally with a cap on
// CTAs per SM: see launch_width) on the caller's own inputs (one warm-up and
// two timed launches each, CUDA events on `s`), keep the fastest.  Candidates
// that cannot launch for this shape, or whose cap would not lower the
// residency, are skipped.
template <typename T>
int tune_signature(const rpp_gb_plan* plan, cudaStream_t s, int32_t dtype, const void* incr, const int64_t* offsets,
                   int64_t length, int64_t batch, void* sig, int64_t sig_stride, const void* seed,
                   int64_t seed_stride, void* grad, int32_t* chosen, float* best_ms_out) {
    if (int rc = check_signature_args<T>(plan, incr, offsets, length, sig, sig_stride, seed, seed_stride, grad,
                                         true))
        return rc;
    static const int sizes[] = {128, 192, 256, 320, 384, 512};
    static const int caps[] = {0, 3, 2};
    int candidates[sizeof(sizes) / sizeof(sizes[0]) * 8 + 64];
    int ncand = 0;
    for (int c : caps)
        for (int t : sizes) candidates[ncand++] = t | (c << 10);
    // forward + reverse with signature output may also run as two launches,
    // optionally with the forward launch's top level in global memory
    if (sig && seed && grad)
        for (int t : sizes) {
            candidates[ncand++] = t | rpp_gb::kScheduleSplit;
            candidates[ncand++] = t | rpp_gb::kScheduleSplit | rpp_gb::kScheduleForwardTopGlobal;
        }
    // a reverse pass with the cotangent arrays in a global workspace (fused
    // form, and the two-launch form's reverse launch)
    if (seed && grad)
        for (int t : {256, 320, 384, 512}) {
            candidates[ncand++] = t | rpp_gb::kScheduleCotangentGlobal;
            if (sig)  // the two-launch form: this forward size with a 512-thread reverse launch too
                for (int rev : {0, 512})
                    candidates[ncand++] = t | rpp_gb::kScheduleSplit | rpp_gb::kScheduleForwardTopGlobal |
                                          rpp_gb::kScheduleCotangentGlobal | (rev << rpp_gb::kScheduleReverseShift);
        }
    // forward-only: the top level in the output row, not in shared memory
    // (more CTAs per SM where the whole state holds only one)
    if (sig && !seed)
        for (int t : sizes) candidates[ncand++] = t | rpp_gb::kScheduleForwardTopGlobal;
    // FP32: the kernels with one warp per first letter (forward-only, and
    // forward + reverse)
    if (std::is_same<T, float>::value &&
        ((sig && !seed && rpp_gb::letter_warps_supported(plan->geometry.width, plan->geometry.depth)) ||
         (seed && rpp_gb::letter_reverse_supported(plan->geometry.width, plan->geometry.depth))))
        candidates[ncand++] = 32 | rpp_gb::kScheduleLetterWarps;
    // a state split over a cluster of P CTAs by first letter (P divides the
    // width), for states whose tensor alone exceeds 48 KB
    const auto& geo = plan->geometry;
    if (static_cast<size_t>(geo.dim) * sizeof(T) > (size_t(48) << 10) && geo.depth >= 2)
        for (int P : {2, 3, 4, 6, 8})
            if (P <= geo.width && geo.width % P == 0)
                for (int t : {256, 512})
                    for (int top : {0, rpp_gb::kScheduleForwardTopGlobal})
                        for (int cot : {0, rpp_gb::kScheduleCotangentGlobal}) {
                            if (cot && !(seed && grad)) continue;
                            candidates[ncand++] = t | top | cot | ((P - 1) << rpp_gb::kScheduleClusterShift);
                        }
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return fail(RPP_GB_OUT_OF_RESOURCES, "cudaEventCreate failed");
    int best = 0;
    float best_ms = 0.f;
    bool device_ok = true;
    // the three fastest candidates so far (ms, schedule), fastest first
    std::pair<float, int> top[3] = {{0.f, 0}, {0.f, 0}, {0.f, 0}};
    // one warm-up and two timed calls of candidate `t`; keeps the fastest
    auto time_candidate = [&](int t, float& ms) -> bool {
        if (!device_ok) return false;
        int rc = RPP_GB_SUCCESS;
        for (int rep = 0; rep < 3 && rc == RPP_GB_SUCCESS; ++rep) {
            if (rep == 1) cudaEventRecord(e0, s);
            rc = run_signature<T>(plan, s, dtype, incr, offsets, length, batch, sig, sig_stride, seed, seed_stride,
                                  grad, true, t);
        }
        if (rc != RPP_GB_SUCCESS) {
            cudaGetLastError();  // configuration errors are not sticky; skip this candidate
            return false;
        }
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            device_ok = false;
            return false;
        }
        cudaEventElapsedTime(&ms, e0, e1);
        return true;
    };
    auto try_candidate = [&](int t) {
        float ms = 0.f;
        if (!time_candidate(t, ms)) return;
        if (best == 0 || ms < best_ms) {
            best = t;
            best_ms = ms;
        }
        for (int k = 0; k < 3; ++k)
            if (top[k].second == t) return;
        for (int k = 0; k < 3; ++k)
            if (top[k].second == 0 || ms < top[k].first) {
                for (int m = 2; m > k; --m) top[m] = top[m - 1];
                top[k] = {ms, t};
                break;
            }
    };
    for (int ci = 0; ci < ncand; ++ci) try_candidate(candidates[ci]);
    // A two-launch winner: its forward and reverse launches may prefer
    // different CTA sizes.  Try other reverse sizes, then other forward sizes
    // with the best reverse size.
    if (best & rpp_gb::kScheduleSplit) {
        constexpr int sh = rpp_gb::kScheduleReverseShift;
        const int fwd = best & 1023;
        const int flags = best & ~1023 & ~(1023 << sh);
        for (int t : sizes)
            if (t != fwd) try_candidate(flags | fwd | (t << sh));
        const int rev = (best >> sh) & 1023 ? (best >> sh) & 1023 : fwd;
        for (int t : sizes)
            if (t != fwd) try_candidate(flags | t | (rev << sh));
    }
    // The D-barrier reverse step (kScheduleMergedReverse) on the three
    // fastest so far (measured: 4 % faster at W16 D3, 1.7 % at W8 D4, equal
    // at W5 D5 and W2 D12, slower with the global workspace at W6 D6).
    if (seed && grad) {
        int base[3];
        for (int k = 0; k < 3; ++k) base[k] = top[k].second;
        for (int k = 0; k < 3; ++k)
            if (base[k] != 0 && ((base[k] >> rpp_gb::kScheduleClusterShift) & 7) == 0 &&
                !((base[k] & rpp_gb::kScheduleLetterWarps) && !(base[k] & rpp_gb::kScheduleSplit)))
                try_candidate(base[k] | rpp_gb::kScheduleMergedReverse);
    }
    // Near-ties are decided by noise in a single timing: time the three
    // fastest once more and keep the best total of both timings.
    if (top[1].second != 0) {
        float best_total = 0.f;
        for (const auto& c : top) {
            float ms = 0.f;
            if (c.second == 0 || !time_candidate(c.second, ms)) continue;
            if (best_total == 0.f || c.first + ms < best_total) {
                best_total = c.first + ms;
                best = c.second;
                best_ms = best_total / 2.f;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best == 0) return fail(RPP_GB_NOT_IMPLEMENTED, "no signature schedule can launch for this shape");
    {
        std::lock_guard<std::mutex> guard(g_schedule_lock);
        g_schedules[schedule_key(plan, dtype, true, sig, seed, offsets)] = best;
    }
    if (chosen) *chosen = best;
    if (best_ms_out) *best_ms_out = best_ms / 2.f;
    // leave the outputs of the chosen schedule in place
    return run_signature<T>(plan, s, dtype, incr, offsets, length, batch, sig, sig_stride, seed, seed_stride, grad,
                            true, best);
}

// Host buffers in, host buffers out: chunks of the batch go round two
// internal streams, each chunk copied in, computed (the recorded schedule of
// this shape, as rpp_gb_signature) and copied out on its stream, so one
// chunk's copies overlap another chunk's kernels.  Paths are independent, so
// the results equal rpp_gb_signature's on device copies of the same arrays.
cudaError_t copy_rows(void* dst, size_t dst_pitch, const void* src, size_t src_pitch, size_t row_bytes, size_t rows,
                      cudaMemcpyKind kind, cudaStream_t s) {
    if (rows == 0) return cudaSuccess;
    if (dst_pitch == row_bytes && src_pitch == row_bytes)
        return cudaMemcpyAsync(dst, src, row_bytes * rows, kind, s);
    return cudaMemcpy2DAsync(dst, dst_pitch, src, src_pitch, row_bytes, rows, kind, s);
}

template <typename T>
int run_signature_host(const rpp_gb_plan* plan, cudaStream_t s, int32_t dtype, const void* incr, int64_t length,
                       int64_t batch, void* sig, int64_t sig_stride, const void* seed, int64_t seed_stride,
                       void* grad, int64_t chunk) {
    const auto& g = plan->geometry;
    if (length <= 0) return fail(RPP_GB_INVALID_ARGUMENT, "host-buffer signatures need equal path lengths > 0");
    if (!incr) return fail(RPP_GB_INVALID_ARGUMENT, "increments are NULL");
    if ((seed == nullptr) != (grad == nullptr)) return fail(RPP_GB_INVALID_ARGUMENT, "seed and grad must be given together");
    if (!sig && !grad) return fail(RPP_GB_INVALID_ARGUMENT, "nothing to compute");
    const int64_t dim = g.dim, row = length * g.width;
    if ((sig && sig_stride < dim) || (seed && seed_stride < dim))
        return fail(RPP_GB_INVALID_ARGUMENT, "stride shorter than the tensor dimension");
    if (chunk <= 0) chunk = (batch + 1) / 2;
    chunk = std::min(chunk, batch);
    const size_t ts = sizeof(T);
    const size_t per_path = static_cast<size_t>(2 * row + (sig ? dim : 0) + (seed ? dim : 0));
    const size_t bytes = per_path * static_cast<size_t>(chunk) * ts;

    cudaStream_t st[2] = {nullptr, nullptr};
    cudaEvent_t ready = nullptr, done[2] = {nullptr, nullptr};
    char* buf[2] = {nullptr, nullptr};
    cudaError_t err = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    for (int i = 0; i < 2 && err == cudaSuccess; ++i) {
        err = cudaStreamCreateWithFlags(&st[i], cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
    }
    if (err == cudaSuccess) err = cudaEventRecord(ready, s);  // after the caller's earlier work
    for (int i = 0; i < 2 && err == cudaSuccess; ++i) {
        err = cudaStreamWaitEvent(st[i], ready, 0);
        if (err == cudaSuccess) err = cudaMallocAsync(reinterpret_cast<void**>(&buf[i]), bytes, st[i]);
    }
    int rc = err == cudaSuccess ? static_cast<int>(RPP_GB_SUCCESS) : cuda_status(err, "host-buffer signature setup");
    for (int64_t b0 = 0, c = 0; b0 < batch && rc == RPP_GB_SUCCESS; b0 += chunk, ++c) {
        const int i = static_cast<int>(c & 1);
        const int64_t nb = std::min(chunk, batch - b0);
        T* d_incr = reinterpret_cast<T*>(buf[i]);
        T* d_grad = grad ? d_incr + chunk * row : nullptr;
        T* d_sig = sig ? d_incr + 2 * chunk * row : nullptr;
        T* d_seed = seed ? d_incr + 2 * chunk * row + (sig ? chunk * dim : 0) : nullptr;
        const auto* h_incr = static_cast<const char*>(incr) + b0 * row * ts;
        err = cudaMemcpyAsync(d_incr, h_incr, static_cast<size_t>(nb * row) * ts, cudaMemcpyHostToDevice, st[i]);
        if (err == cudaSuccess && seed)
            err = copy_rows(d_seed, dim * ts, static_cast<const char*>(seed) + b0 * seed_stride * ts, seed_stride * ts,
                            dim * ts, nb, cudaMemcpyHostToDevice, st[i]);
        if (err != cudaSuccess) {
            rc = cuda_status(err, "host-to-device copy");
            break;
        }
        rc = run_signature<T>(plan, st[i], dtype, d_incr, nullptr, length, nb, d_sig, dim, d_seed, dim, d_grad, true);
        if (rc != RPP_GB_SUCCESS) break;
        if (sig)
            err = copy_rows(static_cast<char*>(sig) + b0 * sig_stride * ts, sig_stride * ts, d_sig, dim * ts, dim * ts,
                            nb, cudaMemcpyDeviceToHost, st[i]);
        if (err == cudaSuccess && grad)
            err = cudaMemcpyAsync(static_cast<char*>(grad) + b0 * row * ts, d_grad, static_cast<size_t>(nb * row) * ts,
                                  cudaMemcpyDeviceToHost, st[i]);
        if (err != cudaSuccess) rc = cuda_status(err, "device-to-host copy");
    }
    // release the buffers after their last use, then order the caller's
    // stream after both internal streams
    for (int i = 0; i < 2; ++i) {
        if (!st[i]) continue;
        if (buf[i]) cudaFreeAsync(buf[i], st[i]);
        if (done[i] && cudaEventRecord(done[i], st[i]) == cudaSuccess) cudaStreamWaitEvent(s, done[i], 0);
    }
    for (int i = 0; i < 2; ++i) {
        if (done[i]) cudaEventDestroy(done[i]);
        if (st[i]) cudaStreamDestroy(st[i]);
    }
    if (ready) cudaEventDestroy(ready);
    return rc;
}

}  // namespace

// Shuffle algebra: operand conversion and order computation shared by the
// entry points below.
template <typename T>
int run_shuffle_product(const rpp_gb_plan* plan, cudaStream_t s, rpp_gb::ShuffleKind kind,
                        const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* add, const rpp_gb_tensor_arg* lhs,
                        const rpp_gb_tensor_arg* rhs, int64_t batch, double alpha, double beta) {
    rpp_gb::TArg<T> o, a, l, r;
    const auto& g = plan->geometry;
    const bool left_half = kind == rpp_gb::ShuffleKind::LeftHalf;
    if (!to_targ(out, g, true, batch, o, kind == rpp_gb::ShuffleKind::InplaceFma ? "a" : "out", true) ||
        !to_targ(add, g, false, batch, a, "a") || !to_targ(lhs, g, true, batch, l, left_half ? "integrator" : "lhs") ||
        !to_targ(rhs, g, true, batch, r, left_half ? "integrand" : "rhs"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    const auto ord = rpp_gb::shuffle_product_order(g, o.lo, o.hi);
    return cuda_status(
        rpp_gb::launch_shuffle_product<T>(g, plan->device, s, kind, o, a, l, r, batch, alpha, beta, ord),
        "shuffle product kernel");
}

int run_shuffle_product_any(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, rpp_gb::ShuffleKind kind,
                            const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* add,
                            const rpp_gb_tensor_arg* lhs, const rpp_gb_tensor_arg* rhs, int64_t batch, double alpha,
                            double beta) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64
                   ? run_shuffle_product<double>(plan, s, kind, out, add, lhs, rhs, batch, alpha, beta)
                   : run_shuffle_product<float>(plan, s, kind, out, add, lhs, rhs, batch, alpha, beta);
    });
}

template <typename T>
int run_shuffle_adjoint(const rpp_gb_plan* plan, cudaStream_t s, rpp_gb::ShuffleAdjKind kind,
                        const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op, const rpp_gb_tensor_arg* arg,
                        int64_t batch, double beta) {
    rpp_gb::TArg<T> o, p, a;
    const auto& g = plan->geometry;
    if (!to_targ(out, g, true, batch, o, "out", true) || !to_targ(op, g, true, batch, p, "op") ||
        !to_targ(arg, g, true, batch, a, "arg"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    // the kernels read the fixed operand through `op` and the cotangent
    // through `arg`: the right adjoint's fixed operand is the integrand
    const bool swap = kind == rpp_gb::ShuffleAdjKind::HalfR;
    const auto& fixed = swap ? a : p;
    const auto& cot = swap ? p : a;
    return cuda_status(rpp_gb::launch_shuffle_adjoint<T>(g, plan->device, s, kind, o, fixed, cot, batch, beta),
                       "shuffle adjoint kernel");
}

int run_shuffle_adjoint_any(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                            rpp_gb::ShuffleAdjKind kind, const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op,
                            const rpp_gb_tensor_arg* arg, int64_t batch, double beta) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_shuffle_adjoint<double>(plan, s, kind, out, op, arg, batch, beta)
                                   : run_shuffle_adjoint<float>(plan, s, kind, out, op, arg, batch, beta);
    });
}

template <typename T>
int run_pairing(const rpp_gb_plan* plan, cudaStream_t s, void* result, const rpp_gb_tensor_arg* f,
                const rpp_gb_tensor_arg* a, int64_t batch) {
    rpp_gb::TArg<T> tf, ta;
    const auto& g = plan->geometry;
    if (!result) return fail(RPP_GB_INVALID_ARGUMENT, "tensor_pairing: result is NULL");
    if (!to_targ(f, g, true, batch, tf, "functional") || !to_targ(a, g, true, batch, ta, "arg"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    return cuda_status(rpp_gb::launch_pairing<T>(g, plan->device, s, static_cast<T*>(result), tf, ta, batch),
                       "pairing kernel");
}


// Fused Lie <-> tensor steps.  When the work tensors exceed shared memory the
// unfused kernels are composed through a stream-ordered scratch batch.
bool degree_view(const rpp_gb::Geometry& g, int32_t lo, int32_t hi, int& vlo, int& vhi) {
    if (lo < 0 || hi < lo || lo > g.depth) return false;
    vlo = lo;
    vhi = std::min<int32_t>(hi, g.depth);
    return true;
}

bool check_vector(const rpp_gb_vector_arg* v, int64_t batch, const char* name) {
    if (!v) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + " is NULL");
        return false;
    }
    if (v->begin < 0 || v->size < 0) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + ": negative view offset or size");
        return false;
    }
    if (!v->data) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + ": NULL data");
        return false;
    }
    if (batch > 1 && v->stride < v->begin + v->size) {
        fail(RPP_GB_INVALID_ARGUMENT, std::string(name) + ": stride shorter than the view");
        return false;
    }
    return true;
}

template <typename T>
int run_log_to_lie(const rpp_gb_plan* plan, const rpp_gb_matrix* matrix, cudaStream_t s,
                   const rpp_gb_vector_arg* out, const rpp_gb_tensor_arg* arg, int lo, int hi, int64_t batch,
                   double alpha) {
    const auto& g = plan->geometry;
    const auto& m = matrix->csr;
    rpp_gb::TArg<T> x;
    if (!to_targ(arg, g, true, batch, x, "arg") || !check_vector(out, batch, "out"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    const int64_t view = static_cast<int64_t>(g.db[hi + 1]) - g.db[lo];
    if (m.rows > out->size) return fail(RPP_GB_OUT_OF_BOUNDS, "matrix has more rows than the output view");
    if (m.cols_dim > view) return fail(RPP_GB_OUT_OF_BOUNDS, "matrix has more columns than the log view");
    T* o = static_cast<T*>(out->data) + out->begin;
    // The fused kernel holds two tensors per CTA.  Where only one CTA of it
    // fits per SM its Horner rounds and long t2l rows find nothing to overlap
    // with, and ft_log + SpMM as two launches (through a batch-sized scratch
    // tensor) run faster: W2 D12 FP64, 16 384 tensors, 14.5 ms fused against
    // 8.0 + 4.4 ms.  So the fused kernel runs where two CTAs fit per SM.
    if (2 * rpp_gb::log_to_lie_smem(g, sizeof(T)) <= static_cast<size_t>(plan->device.max_smem_optin))
        return cuda_status(rpp_gb::launch_log_to_lie<T>(g, plan->device, s, m, x, lo, hi, o, out->stride, out->size,
                                                        batch, alpha),
                           "log-to-Lie kernel");
    T* tmp = nullptr;
    const size_t bytes = static_cast<size_t>(batch) * g.dim * sizeof(T);
    cudaError_t err = cudaMallocAsync(reinterpret_cast<void**>(&tmp), bytes, s);
    if (err != cudaSuccess) return cuda_status(err, "log-to-Lie scratch");
    rpp_gb::TArg<T> t{tmp, static_cast<int64_t>(g.dim), lo, hi};
    err = rpp_gb::launch_intermediate<T>(g, plan->device, s, rpp_gb::IntermediateKind::Log, t, x, rpp_gb::TArg<T>{},
                                         batch);
    if (err == cudaSuccess)
        err = rpp_gb::launch_spmm<T>(m, plan->device, s, o, out->stride, out->size, tmp + g.db[lo], g.dim, view, batch,
                                     alpha);
    const cudaError_t ferr = cudaFreeAsync(tmp, s);
    return cuda_status(err != cudaSuccess ? err : ferr, "log-to-Lie (composed)");
}

template <typename T>
int run_lie_exp(const rpp_gb_plan* plan, const rpp_gb_matrix* matrix, cudaStream_t s, const rpp_gb_tensor_arg* out,
                const rpp_gb_tensor_arg* mult, const rpp_gb_vector_arg* arg, int lo, int hi, int64_t batch,
                double alpha) {
    const auto& g = plan->geometry;
    const auto& m = matrix->csr;
    rpp_gb::TArg<T> o, mm;
    if (!to_targ(out, g, true, batch, o, "out", true) || !to_targ(mult, g, false, batch, mm, "multiplier") ||
        !check_vector(arg, batch, "arg"))
        return static_cast<int>(RPP_GB_INVALID_ARGUMENT);
    if (mult && out->data == mult->data) return fail(RPP_GB_INVALID_ARGUMENT, "out must not alias multiplier");
    const int64_t view = static_cast<int64_t>(g.db[hi + 1]) - g.db[lo];
    if (m.rows > view) return fail(RPP_GB_OUT_OF_BOUNDS, "matrix has more rows than the tensor view");
    if (m.cols_dim > arg->size) return fail(RPP_GB_OUT_OF_BOUNDS, "matrix has more columns than the argument view");
    const T* lie = static_cast<const T*>(arg->data) + arg->begin;
    if (rpp_gb::lie_exp_smem(g, sizeof(T), mult != nullptr) <= static_cast<size_t>(plan->device.max_smem_optin) &&
        m.cols_dim <= static_cast<int64_t>(g.dim))
        return cuda_status(
            rpp_gb::launch_lie_exp<T>(g, plan->device, s, m, lie, arg->stride, lo, hi, o, mm, batch, alpha),
            "Lie-exp kernel");
    T* tmp = nullptr;
    const size_t bytes = static_cast<size_t>(batch) * g.dim * sizeof(T);
    cudaError_t err = cudaMallocAsync(reinterpret_cast<void**>(&tmp), bytes, s);
    if (err != cudaSuccess) return cuda_status(err, "Lie-exp scratch");
    err = cudaMemsetAsync(tmp, 0, bytes, s);
    if (err == cudaSuccess)
        err = rpp_gb::launch_spmm<T>(m, plan->device, s, tmp + g.db[lo], g.dim, view, lie, arg->stride, arg->size,
                                     batch, alpha);
    if (err == cudaSuccess) {
        rpp_gb::TArg<T> t{tmp, static_cast<int64_t>(g.dim), std::max(1, lo), hi};
        err = rpp_gb::launch_intermediate<T>(g, plan->device, s,
                                             mult ? rpp_gb::IntermediateKind::FMExp : rpp_gb::IntermediateKind::Exp,
                                             o, t, mm, batch);
    }
    const cudaError_t ferr = cudaFreeAsync(tmp, s);
    return cuda_status(err != cudaSuccess ? err : ferr, "Lie-exp (composed)");
}

template <typename F>
int with_plan_matrix(const rpp_gb_plan* plan, const rpp_gb_matrix* matrix, int32_t dtype, int64_t batch,
                     int32_t min_degree, int32_t max_degree, int& lo, int& hi, F&& body) {
    if (!matrix) return fail(RPP_GB_INVALID_ARGUMENT, "matrix is NULL");
    if (plan && matrix->device != plan->device.device)
        return fail(RPP_GB_INVALID_ARGUMENT, "matrix and plan live on different devices");
    if (plan && !degree_view(plan->geometry, min_degree, max_degree, lo, hi))
        return fail(RPP_GB_INVALID_ARGUMENT, "degree range must satisfy 0 <= min <= max, min <= depth");
    return with_plan(plan, dtype, batch, std::forward<F>(body));
}


extern "C" {

const char* rpp_gb_last_error_string(void) { return g_last_error.c_str(); }

const char* rpp_gb_version(void) { return "rpp_gb300 1.0.0 sm_103a"; }

int rpp_gb_plan_create(rpp_gb_plan** plan, int32_t width, int32_t depth, int32_t device) {
    if (!plan) return fail(RPP_GB_INVALID_ARGUMENT, "plan output pointer is NULL");
    *plan = nullptr;
    if (width < 1 || width > 255) return fail(RPP_GB_INVALID_ARGUMENT, "width must be in [1, 255]");
    if (depth < 0 || depth > rpp_gb::kMaxDepth) return fail(RPP_GB_INVALID_ARGUMENT, "depth must be in [0, 30]");
    rpp_gb::Geometry g{};
    g.width = width;
    g.depth = depth;
    uint64_t db = 0, pw = 1;
    for (int32_t n = 0; n <= depth; ++n) {
        g.db[n] = static_cast<uint32_t>(db);
        g.pw[n] = static_cast<uint32_t>(pw);
        db += pw;
        if (db >= (uint64_t{1} << 31)) return fail(RPP_GB_OUT_OF_BOUNDS, "tensor dimension must stay below 2^31");
        pw *= static_cast<uint64_t>(width);
    }
    g.db[depth + 1] = static_cast<uint32_t>(db);
    g.pw[depth + 1] = 0;
    g.dim = static_cast<uint32_t>(db);
    g.divw = rpp_gb::FastDiv(static_cast<uint32_t>(width));

    int count = 0;
    cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess) return cuda_status(err, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return fail(RPP_GB_INVALID_ARGUMENT, "no such CUDA device");
    rpp_gb::DeviceInfo info{};
    info.device = device;
    if ((err = cudaDeviceGetAttribute(&info.sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
        return cuda_status(err, "cudaDeviceGetAttribute");
    if ((err = cudaDeviceGetAttribute(&info.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device)) !=
        cudaSuccess)
        return cuda_status(err, "cudaDeviceGetAttribute");
    // the fault word kernels report expired bounded waits in
    uint32_t* fault = nullptr;
    {
        DeviceGuard guard(device);
        if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");
        if ((err = cudaMalloc(reinterpret_cast<void**>(&fault), sizeof(uint32_t))) != cudaSuccess)
            return cuda_status(err, "plan fault word");
        if ((err = cudaMemset(fault, 0, sizeof(uint32_t))) != cudaSuccess) {
            cudaFree(fault);
            return cuda_status(err, "plan fault word");
        }
    }
    g.fault = fault;
    auto* p = new (std::nothrow) rpp_gb_plan;
    if (!p) {
        cudaFree(fault);
        return fail(RPP_GB_OUT_OF_RESOURCES, "out of host memory");
    }
    p->geometry = g;
    p->device = info;
    *plan = p;
    return ok();
}

int rpp_gb_plan_destroy(rpp_gb_plan* plan) {
    if (plan && plan->geometry.fault) {
        DeviceGuard guard(plan->device.device);
        cudaFree(plan->geometry.fault);
    }
    delete plan;
    return ok();
}

int rpp_gb_plan_fault(const rpp_gb_plan* plan, uint32_t* fault) {
    if (!plan || !fault) return fail(RPP_GB_INVALID_ARGUMENT, "NULL plan or output");
    DeviceGuard guard(plan->device.device);
    if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");
    cudaError_t err = cudaMemcpy(fault, plan->geometry.fault, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemset(plan->geometry.fault, 0, sizeof(uint32_t));
    return cuda_status(err, "plan fault word");
}

int rpp_gb_selftest_bounded_wait(const rpp_gb_plan* plan, rpp_gb_stream stream) {
    if (!plan) return fail(RPP_GB_INVALID_ARGUMENT, "plan is NULL");
    DeviceGuard guard(plan->device.device);
    if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");
    return cuda_status(rpp_gb::launch_expired_wait(plan->geometry, static_cast<cudaStream_t>(stream)),
                       "bounded-wait self-test");
}

int rpp_gb_ft_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                  const rpp_gb_tensor_arg* lhs, const rpp_gb_tensor_arg* rhs, int64_t batch, double beta) {
    return run_product_any(plan, stream, dtype, rpp_gb::ProductKind::Fma, out, nullptr, lhs, rhs, batch, 0.0, beta,
                           false);
}

int rpp_gb_ft_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                  const rpp_gb_tensor_arg* a, const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t batch,
                  double alpha, double beta) {
    return run_product_any(plan, stream, dtype, rpp_gb::ProductKind::Fma, out, a, b, c, batch, alpha, beta, true);
}

int rpp_gb_ft_inplace_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, int32_t kind,
                          const rpp_gb_tensor_arg* a, const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c,
                          int64_t batch, double alpha, double beta) {
    rpp_gb::ProductKind k;
    switch (kind) {
        case RPP_GB_A_EQUALS_BC_PLUS_A: k = rpp_gb::ProductKind::InplaceBCA; break;
        case RPP_GB_A_EQUALS_AB_PLUS_C: k = rpp_gb::ProductKind::InplaceABC; break;
        case RPP_GB_A_EQUALS_BA_PLUS_C: k = rpp_gb::ProductKind::InplaceBAC; break;
        default: return fail(RPP_GB_INVALID_ARGUMENT, "unknown in-place FMA kind");
    }
    return run_product_any(plan, stream, dtype, k, a, nullptr, b, c, batch, alpha, beta, false);
}

int rpp_gb_ft_inplace_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          const rpp_gb_tensor_arg* lhs, const rpp_gb_tensor_arg* rhs, int64_t batch, double beta) {
    return run_product_any(plan, stream, dtype, rpp_gb::ProductKind::InplaceMul, lhs, nullptr, rhs, nullptr, batch,
                           0.0, beta, false);
}

int rpp_gb_ft_exp(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                  const rpp_gb_tensor_arg* arg, int64_t batch) {
    return run_intermediate_any(plan, stream, dtype, rpp_gb::IntermediateKind::Exp, out, arg, nullptr, batch);
}

int rpp_gb_ft_fmexp(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                    const rpp_gb_tensor_arg* multiplier, const rpp_gb_tensor_arg* exponent, int64_t batch) {
    return run_intermediate_any(plan, stream, dtype, rpp_gb::IntermediateKind::FMExp, out, exponent, multiplier,
                                batch);
}

int rpp_gb_ft_log(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                  const rpp_gb_tensor_arg* arg, int64_t batch) {
    return run_intermediate_any(plan, stream, dtype, rpp_gb::IntermediateKind::Log, out, arg, nullptr, batch);
}

int rpp_gb_ft_adj_lmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                       const rpp_gb_tensor_arg* op, const rpp_gb_tensor_arg* arg, int64_t batch) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_adjoint<double>(plan, s, true, out, op, arg, batch)
                                   : run_adjoint<float>(plan, s, true, out, op, arg, batch);
    });
}

int rpp_gb_ft_adj_rmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                       const rpp_gb_tensor_arg* op, const rpp_gb_tensor_arg* arg, int64_t batch) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_adjoint<double>(plan, s, false, out, op, arg, batch)
                                   : run_adjoint<float>(plan, s, false, out, op, arg, batch);
    });
}

int rpp_gb_st_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                  const rpp_gb_tensor_arg* lhs, const rpp_gb_tensor_arg* rhs, int64_t batch, double beta) {
    return run_shuffle_product_any(plan, stream, dtype, rpp_gb::ShuffleKind::Mul, out, nullptr, lhs, rhs, batch, 0.0,
                                   beta);
}

int rpp_gb_st_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                  const rpp_gb_tensor_arg* a, const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t batch,
                  double alpha, double beta) {
    return run_shuffle_product_any(plan, stream, dtype, rpp_gb::ShuffleKind::Fma, out, a, b, c, batch, alpha, beta);
}

int rpp_gb_st_inplace_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* a,
                          const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t batch, double alpha,
                          double beta) {
    return run_shuffle_product_any(plan, stream, dtype, rpp_gb::ShuffleKind::InplaceFma, a, nullptr, b, c, batch,
                                   alpha, beta);
}

int rpp_gb_st_adj_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                      const rpp_gb_tensor_arg* op, const rpp_gb_tensor_arg* arg, int64_t batch) {
    return run_shuffle_adjoint_any(plan, stream, dtype, rpp_gb::ShuffleAdjKind::Shuffle, out, op, arg, batch, 1.0);
}

int rpp_gb_left_hs_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                       const rpp_gb_tensor_arg* integrator, const rpp_gb_tensor_arg* integrand, int64_t batch,
                       double beta) {
    return run_shuffle_product_any(plan, stream, dtype, rpp_gb::ShuffleKind::LeftHalf, out, nullptr, integrator,
                                   integrand, batch, 0.0, beta);
}

int rpp_gb_left_hs_adj_lmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                            const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op, const rpp_gb_tensor_arg* arg,
                            int64_t batch, double beta) {
    return run_shuffle_adjoint_any(plan, stream, dtype, rpp_gb::ShuffleAdjKind::HalfL, out, op, arg, batch, beta);
}

int rpp_gb_left_hs_adj_rmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                            const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op, const rpp_gb_tensor_arg* arg,
                            int64_t batch, double beta) {
    return run_shuffle_adjoint_any(plan, stream, dtype, rpp_gb::ShuffleAdjKind::HalfR, out, op, arg, batch, beta);
}

int rpp_gb_tensor_pairing(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, void* result,
                          const rpp_gb_tensor_arg* functional, const rpp_gb_tensor_arg* arg, int64_t batch) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_pairing<double>(plan, s, result, functional, arg, batch)
                                   : run_pairing<float>(plan, s, result, functional, arg, batch);
    });
}

int rpp_gb_tensor_antipode(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, int32_t policy,
                           const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* arg, int64_t batch) {
    if (policy != RPP_GB_NO_SIGNING && policy != RPP_GB_SIGN_BY_DEGREE)
        return fail(RPP_GB_INVALID_ARGUMENT, "unknown antipode signing policy");
    return with_plan(plan, dtype, batch, [&]() -> int {
        auto s = static_cast<cudaStream_t>(stream);
        const auto& g = plan->geometry;
        const bool sign = policy == RPP_GB_SIGN_BY_DEGREE;
        if (dtype == RPP_GB_F64) {
            rpp_gb::TArg<double> o, a;
            if (!to_targ(out, g, true, batch, o, "out", true) || !to_targ(arg, g, true, batch, a, "arg"))
                return RPP_GB_INVALID_ARGUMENT;
            return cuda_status(rpp_gb::launch_antipode<double>(g, plan->device, s, sign, o, a, batch), "antipode");
        }
        rpp_gb::TArg<float> o, a;
        if (!to_targ(out, g, true, batch, o, "out", true) || !to_targ(arg, g, true, batch, a, "arg"))
            return RPP_GB_INVALID_ARGUMENT;
        return cuda_status(rpp_gb::launch_antipode<float>(g, plan->device, s, sign, o, a, batch), "antipode");
    });
}

int rpp_gb_vector_assign(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const rpp_gb_tensor_arg* out,
                         const rpp_gb_tensor_arg* arg, int64_t batch) {
    return run_helper_any(plan, stream, dtype, rpp_gb::HelperKind::Assign, out, arg, batch, 0.0);
}

int rpp_gb_vector_set_constant(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                               const rpp_gb_tensor_arg* out, int64_t batch, double value) {
    return run_helper_any(plan, stream, dtype, rpp_gb::HelperKind::SetConstant, out, nullptr, batch, value);
}

int rpp_gb_tensor_set_identity(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                               const rpp_gb_tensor_arg* out, int64_t batch, double scalar) {
    return run_helper_any(plan, stream, dtype, rpp_gb::HelperKind::SetIdentity, out, nullptr, batch, scalar);
}

int rpp_gb_tensor_add_identity(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                               const rpp_gb_tensor_arg* out, int64_t batch, double scalar) {
    return run_helper_any(plan, stream, dtype, rpp_gb::HelperKind::AddIdentity, out, nullptr, batch, scalar);
}

int rpp_gb_matrix_create(rpp_gb_matrix** matrix, int32_t format, int64_t outer_dim, int64_t inner_dim, int64_t nnz,
                         const int64_t* offsets, const int64_t* indices, const double* values, int32_t device) {
    if (!matrix) return fail(RPP_GB_INVALID_ARGUMENT, "matrix output pointer is NULL");
    *matrix = nullptr;
    if (format != RPP_GB_CSR && format != RPP_GB_CSC) return fail(RPP_GB_INVALID_ARGUMENT, "unknown matrix format");
    if (outer_dim < 0 || inner_dim < 0 || nnz < 0) return fail(RPP_GB_INVALID_ARGUMENT, "negative matrix size");
    if (nnz > std::numeric_limits<int32_t>::max() || outer_dim >= std::numeric_limits<int32_t>::max() ||
        inner_dim >= std::numeric_limits<int32_t>::max())
        return fail(RPP_GB_OUT_OF_BOUNDS, "matrix too large for 32-bit indices");
    if (!offsets || (nnz > 0 && (!indices || !values))) return fail(RPP_GB_INVALID_ARGUMENT, "NULL matrix arrays");
    if (offsets[0] != 0 || offsets[outer_dim] != nnz)
        return fail(RPP_GB_INVALID_ARGUMENT, "offsets must start at 0 and end at nnz");
    for (int64_t o = 0; o < outer_dim; ++o)
        if (offsets[o + 1] < offsets[o]) return fail(RPP_GB_INVALID_ARGUMENT, "offsets must be non-decreasing");
    for (int64_t e = 0; e < nnz; ++e)
        if (indices[e] < 0 || indices[e] >= inner_dim)
            return fail(RPP_GB_OUT_OF_BOUNDS, "matrix index outside the inner dimension");

    // CSR on the host: rows, row offsets, column indices, values.
    const int64_t rows = format == RPP_GB_CSR ? outer_dim : inner_dim;
    const int64_t cols = format == RPP_GB_CSR ? inner_dim : outer_dim;
    std::vector<int32_t> roff(static_cast<size_t>(rows) + 1, 0), rcol(static_cast<size_t>(nnz));
    std::vector<double> rval(static_cast<size_t>(nnz));
    if (format == RPP_GB_CSR) {
        for (int64_t r = 0; r <= rows; ++r) roff[r] = static_cast<int32_t>(offsets[r]);
        for (int64_t e = 0; e < nnz; ++e) {
            rcol[e] = static_cast<int32_t>(indices[e]);
            rval[e] = values[e];
        }
    } else {
        // Transpose (the reference's swap_format): entries of a row keep
        // ascending column order.
        for (int64_t e = 0; e < nnz; ++e) ++roff[static_cast<size_t>(indices[e]) + 1];
        for (int64_t r = 0; r < rows; ++r) roff[r + 1] += roff[r];
        std::vector<int32_t> pos(roff.begin(), roff.end() - 1);
        for (int64_t c = 0; c < cols; ++c)
            for (int64_t e = offsets[c]; e < offsets[c + 1]; ++e) {
                const int32_t dst = pos[static_cast<size_t>(indices[e])]++;
                rcol[dst] = static_cast<int32_t>(c);
                rval[dst] = values[e];
            }
    }
    std::vector<float> rval32(rval.begin(), rval.end());

    // Sliced ELL copy (CsrDevice): rows by decreasing length, 32 per slice,
    // entry-major within a slice.
    std::vector<int32_t> rord(static_cast<size_t>(rows)), rlen(static_cast<size_t>(rows));
    for (int64_t r = 0; r < rows; ++r) rord[r] = static_cast<int32_t>(r);
    std::stable_sort(rord.begin(), rord.end(), [&](int32_t a, int32_t b) {
        return roff[a + 1] - roff[a] > roff[b + 1] - roff[b];
    });
    const int64_t nslices = (rows + 31) / 32;
    std::vector<int32_t> soff(static_cast<size_t>(nslices) + 1, 0);
    int64_t ell_total = 0;
    for (int64_t i = 0; i < rows; ++i) rlen[i] = roff[rord[i] + 1] - roff[rord[i]];
    for (int64_t s = 0; s < nslices; ++s) {
        ell_total += 32 * static_cast<int64_t>(rlen[static_cast<size_t>(32 * s)]);  // its longest row
        if (ell_total > std::numeric_limits<int32_t>::max())
            return fail(RPP_GB_OUT_OF_BOUNDS, "matrix too large for 32-bit sliced indices");
        soff[s + 1] = static_cast<int32_t>(ell_total);
    }
    std::vector<int32_t> ecol(static_cast<size_t>(ell_total), 0);
    std::vector<double> ev64(static_cast<size_t>(ell_total), 0.0);
    for (int64_t i = 0; i < rows; ++i) {
        const int64_t base = soff[static_cast<size_t>(i / 32)] + i % 32;
        const int32_t r = rord[i];
        for (int32_t k = 0; k < rlen[i]; ++k) {
            ecol[base + 32 * k] = rcol[roff[r] + k];
            ev64[base + 32 * k] = rval[roff[r] + k];
        }
    }
    std::vector<float> ev32(ev64.begin(), ev64.end());

    int count = 0;
    cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess) return cuda_status(err, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return fail(RPP_GB_INVALID_ARGUMENT, "no such CUDA device");
    DeviceGuard guard(device);
    if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");

    auto align = [](size_t n) { return (n + 255) & ~size_t(255); };
    const size_t b_off = align(roff.size() * sizeof(int32_t));
    const size_t b_col = align(std::max<size_t>(1, rcol.size()) * sizeof(int32_t));
    const size_t b_v64 = align(std::max<size_t>(1, rval.size()) * sizeof(double));
    const size_t b_v32 = align(std::max<size_t>(1, rval32.size()) * sizeof(float));
    const size_t b_fault = 256;  // the fault word of the SpMM's bounded waits
    const size_t b_ord = align(std::max<size_t>(1, rord.size()) * sizeof(int32_t));
    const size_t b_soff = align(soff.size() * sizeof(int32_t));
    const size_t b_ecol = align(std::max<size_t>(1, ecol.size()) * sizeof(int32_t));
    const size_t b_ev64 = align(std::max<size_t>(1, ev64.size()) * sizeof(double));
    const size_t b_ev32 = align(std::max<size_t>(1, ev32.size()) * sizeof(float));
    const size_t b_csr = b_off + b_col + b_v64 + b_v32 + b_fault;
    char* block = nullptr;
    if ((err = cudaMalloc(&block, b_csr + 2 * b_ord + b_soff + b_ecol + b_ev64 + b_ev32)) != cudaSuccess)
        return cuda_status(err, "cudaMalloc");
    auto* m = new (std::nothrow) rpp_gb_matrix;
    if (!m) {
        cudaFree(block);
        return fail(RPP_GB_OUT_OF_RESOURCES, "out of host memory");
    }
    m->allocation = block;
    m->device = device;
    auto* d_off = reinterpret_cast<int32_t*>(block);
    auto* d_col = reinterpret_cast<int32_t*>(block + b_off);
    auto* d_v64 = reinterpret_cast<double*>(block + b_off + b_col);
    auto* d_v32 = reinterpret_cast<float*>(block + b_off + b_col + b_v64);
    auto* d_fault = reinterpret_cast<uint32_t*>(block + b_off + b_col + b_v64 + b_v32);
    char* sell = block + b_csr;
    auto* d_ord = reinterpret_cast<int32_t*>(sell);
    auto* d_len = reinterpret_cast<int32_t*>(sell + b_ord);
    auto* d_soff = reinterpret_cast<int32_t*>(sell + 2 * b_ord);
    auto* d_ecol = reinterpret_cast<int32_t*>(sell + 2 * b_ord + b_soff);
    auto* d_ev64 = reinterpret_cast<double*>(sell + 2 * b_ord + b_soff + b_ecol);
    auto* d_ev32 = reinterpret_cast<float*>(sell + 2 * b_ord + b_soff + b_ecol + b_ev64);
    if ((err = cudaMemset(d_fault, 0, sizeof(uint32_t))) != cudaSuccess) {
        cudaFree(block);
        delete m;
        return cuda_status(err, "cudaMemset");
    }
    err = cudaMemcpy(d_off, roff.data(), roff.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (err == cudaSuccess && nnz > 0) err = cudaMemcpy(d_col, rcol.data(), rcol.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (err == cudaSuccess && nnz > 0) err = cudaMemcpy(d_v64, rval.data(), rval.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (err == cudaSuccess && nnz > 0) err = cudaMemcpy(d_v32, rval32.data(), rval32.size() * sizeof(float), cudaMemcpyHostToDevice);
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (err == cudaSuccess && bytes > 0) err = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    up(d_ord, rord.data(), rord.size() * sizeof(int32_t));
    up(d_len, rlen.data(), rlen.size() * sizeof(int32_t));
    up(d_soff, soff.data(), soff.size() * sizeof(int32_t));
    up(d_ecol, ecol.data(), ecol.size() * sizeof(int32_t));
    up(d_ev64, ev64.data(), ev64.size() * sizeof(double));
    up(d_ev32, ev32.data(), ev32.size() * sizeof(float));
    if (err != cudaSuccess) {
        cudaFree(block);
        delete m;
        return cuda_status(err, "cudaMemcpy");
    }
    m->csr = rpp_gb::CsrDevice{d_off,  d_col, d_v64,  d_v32, rows,   cols,   nnz,  format == RPP_GB_CSC,
                               d_fault, d_ord, d_len, d_soff, d_ecol, d_ev64, d_ev32};
    *matrix = m;
    return ok();
}

int rpp_gb_matrix_destroy(rpp_gb_matrix* matrix) {
    if (!matrix) return ok();
    DeviceGuard guard(matrix->device);
    cudaError_t err = cudaFree(matrix->allocation);
    delete matrix;
    return cuda_status(err, "cudaFree");
}

int rpp_gb_sparse_matrix_vector(const rpp_gb_matrix* matrix, rpp_gb_stream stream, int32_t dtype,
                                const rpp_gb_vector_arg* out, const rpp_gb_vector_arg* arg, int64_t batch,
                                double alpha) {
    if (!matrix || !out || !arg) return fail(RPP_GB_INVALID_ARGUMENT, "NULL matrix or operand");
    if (!valid_dtype(dtype)) return fail(RPP_GB_INVALID_ARGUMENT, "unknown dtype");
    if (batch < 0) return fail(RPP_GB_INVALID_ARGUMENT, "negative batch size");
    if (batch == 0) return ok();
    const auto& m = matrix->csr;
    if (out->begin < 0 || arg->begin < 0 || out->size < 0 || arg->size < 0)
        return fail(RPP_GB_INVALID_ARGUMENT, "negative view offset or size");
    if (m.rows > out->size) return fail(RPP_GB_OUT_OF_BOUNDS, "matrix has more rows than the output view");
    if (m.cols_dim > arg->size) return fail(RPP_GB_OUT_OF_BOUNDS, "matrix has more columns than the argument view");
    if (!out->data || !arg->data) return fail(RPP_GB_INVALID_ARGUMENT, "NULL vector data");
    if (batch > 1 && (out->stride < out->begin + out->size || arg->stride < arg->begin + arg->size))
        return fail(RPP_GB_INVALID_ARGUMENT, "vector stride shorter than the view");
    DeviceGuard guard(matrix->device);
    if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");
    rpp_gb::DeviceInfo dev{};
    dev.device = matrix->device;
    cudaDeviceGetAttribute(&dev.sm_count, cudaDevAttrMultiProcessorCount, dev.device);
    cudaDeviceGetAttribute(&dev.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev.device);
    auto s = static_cast<cudaStream_t>(stream);
    cudaError_t err;
    if (dtype == RPP_GB_F64)
        err = rpp_gb::launch_spmm<double>(m, dev, s, static_cast<double*>(out->data) + out->begin, out->stride,
                                          out->size, static_cast<const double*>(arg->data) + arg->begin,
                                          arg->stride, arg->size, batch, alpha);
    else
        err = rpp_gb::launch_spmm<float>(m, dev, s, static_cast<float*>(out->data) + out->begin, out->stride,
                                         out->size, static_cast<const float*>(arg->data) + arg->begin, arg->stride,
                                         arg->size, batch, alpha);
    return cuda_status(err, "spmm kernel");
}

int rpp_gb_log_to_lie(const rpp_gb_plan* plan, const rpp_gb_matrix* matrix, rpp_gb_stream stream, int32_t dtype,
                      const rpp_gb_vector_arg* out, const rpp_gb_tensor_arg* arg, int32_t min_degree,
                      int32_t max_degree, int64_t batch, double alpha) {
    int lo = 0, hi = -1;
    return with_plan_matrix(plan, matrix, dtype, batch, min_degree, max_degree, lo, hi, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_log_to_lie<double>(plan, matrix, s, out, arg, lo, hi, batch, alpha)
                                   : run_log_to_lie<float>(plan, matrix, s, out, arg, lo, hi, batch, alpha);
    });
}

int rpp_gb_lie_to_tensor_exp(const rpp_gb_plan* plan, const rpp_gb_matrix* matrix, rpp_gb_stream stream,
                             int32_t dtype, const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* multiplier,
                             const rpp_gb_vector_arg* arg, int32_t min_degree, int32_t max_degree, int64_t batch,
                             double alpha) {
    int lo = 0, hi = -1;
    return with_plan_matrix(plan, matrix, dtype, batch, min_degree, max_degree, lo, hi, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64
                   ? run_lie_exp<double>(plan, matrix, s, out, multiplier, arg, lo, hi, batch, alpha)
                   : run_lie_exp<float>(plan, matrix, s, out, multiplier, arg, lo, hi, batch, alpha);
    });
}

int rpp_gb_matrix_fault(const rpp_gb_matrix* matrix, uint32_t* fault) {
    if (!matrix || !fault) return fail(RPP_GB_INVALID_ARGUMENT, "NULL matrix or output");
    DeviceGuard guard(matrix->device);
    if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");
    cudaError_t err = cudaMemcpy(fault, matrix->csr.fault, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemset(matrix->csr.fault, 0, sizeof(uint32_t));
    return cuda_status(err, "matrix fault word");
}

int rpp_gb_lie_basis(int32_t width, int32_t depth, int64_t* true_size, int64_t* degree_begin, int64_t* pairs) {
    if (width < 1 || width > 255 || depth < 0 || depth > rpp_gb::kMaxDepth)
        return fail(RPP_GB_INVALID_ARGUMENT, "width must be in [1, 255] and depth in [0, 30]");
    try {
        const auto h = rpp_gb::build_hall_basis(width, depth);
        if (true_size) *true_size = h.true_size();
        if (degree_begin) std::copy(h.degree_begin.begin(), h.degree_begin.end(), degree_begin);
        if (pairs) std::copy(h.pairs.begin(), h.pairs.end(), pairs);
    } catch (const std::bad_alloc&) {
        return fail(RPP_GB_OUT_OF_RESOURCES, "out of host memory");
    }
    return ok();
}

int rpp_gb_conversion_matrix(int32_t width, int32_t depth, int32_t which, int64_t* outer_dim, int64_t* inner_dim,
                             int64_t* nnz, int64_t* offsets, int64_t* indices, double* values) {
    if (width < 1 || width > 255 || depth < 0 || depth > rpp_gb::kMaxDepth)
        return fail(RPP_GB_INVALID_ARGUMENT, "width must be in [1, 255] and depth in [0, 30]");
    if (which != 0 && which != 1) return fail(RPP_GB_INVALID_ARGUMENT, "which must be 0 (t2l) or 1 (l2t)");
    try {
        const auto h = rpp_gb::build_hall_basis(width, depth);
        const auto m = rpp_gb::build_conversion_matrix(h, which);
        if (outer_dim) *outer_dim = m.outer_dim;
        if (inner_dim) *inner_dim = m.inner_dim;
        if (nnz) *nnz = static_cast<int64_t>(m.indices.size());
        if (offsets) std::copy(m.offsets.begin(), m.offsets.end(), offsets);
        if (indices) std::copy(m.indices.begin(), m.indices.end(), indices);
        if (values) std::copy(m.values.begin(), m.values.end(), values);
    } catch (const std::bad_alloc&) {
        return fail(RPP_GB_OUT_OF_RESOURCES, "out of host memory");
    }
    return ok();
}

int rpp_gb_exp_letter_vjp(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const void* cotangent,
                          int64_t cotangent_stride, const void* x, int64_t x_stride, void* dx, int64_t dx_stride,
                          int64_t batch) {
    return with_plan(plan, dtype, batch, [&]() -> int {
        const auto& g = plan->geometry;
        if (!cotangent || !x || !dx) return fail(RPP_GB_INVALID_ARGUMENT, "NULL operand");
        if ((batch > 1 && (cotangent_stride < static_cast<int64_t>(g.dim) || x_stride < g.width ||
                           dx_stride < g.width)) ||
            cotangent_stride < 0 || x_stride < 0 || dx_stride < 0)
            return fail(RPP_GB_INVALID_ARGUMENT, "stride shorter than the operand");
        auto s = static_cast<cudaStream_t>(stream);
        cudaError_t err =
            dtype == RPP_GB_F64
                ? rpp_gb::launch_exp_letter_vjp<double>(g, plan->device, s, static_cast<const double*>(cotangent),
                                                        cotangent_stride, static_cast<const double*>(x), x_stride,
                                                        static_cast<double*>(dx), dx_stride, batch)
                : rpp_gb::launch_exp_letter_vjp<float>(g, plan->device, s, static_cast<const float*>(cotangent),
                                                       cotangent_stride, static_cast<const float*>(x), x_stride,
                                                       static_cast<float*>(dx), dx_stride, batch);
        return cuda_status(err, "exp vjp kernel");
    });
}

int rpp_gb_signature(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const void* incr,
                     const int64_t* offsets, int64_t length, int64_t batch, void* sig, int64_t sig_stride,
                     const void* seed, int64_t seed_stride, void* grad) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_signature<double>(plan, s, dtype, incr, offsets, length, batch, sig,
                                                           sig_stride, seed, seed_stride, grad, true)
                                   : run_signature<float>(plan, s, dtype, incr, offsets, length, batch, sig,
                                                          sig_stride, seed, seed_stride, grad, true);
    });
}

int rpp_gb_signature_backward(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const void* incr,
                              const int64_t* offsets, int64_t length, int64_t batch, const void* sig,
                              int64_t sig_stride, const void* seed, int64_t seed_stride, void* grad) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64
                   ? run_signature<double>(plan, s, dtype, incr, offsets, length, batch, const_cast<void*>(sig),
                                           sig_stride, seed, seed_stride, grad, false)
                   : run_signature<float>(plan, s, dtype, incr, offsets, length, batch, const_cast<void*>(sig),
                                          sig_stride, seed, seed_stride, grad, false);
    });
}

int rpp_gb_signature_host(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const void* incr,
                          int64_t length, int64_t batch, void* sig, int64_t sig_stride, const void* seed,
                          int64_t seed_stride, void* grad, int64_t chunk) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_signature_host<double>(plan, s, dtype, incr, length, batch, sig, sig_stride,
                                                                seed, seed_stride, grad, chunk)
                                   : run_signature_host<float>(plan, s, dtype, incr, length, batch, sig, sig_stride,
                                                               seed, seed_stride, grad, chunk);
    });
}

// Same computation as rpp_gb_signature without any device allocation; see
// the header and signature.cu for who needs it and its limits.
int rpp_gb_signature_static_scratch(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const void* incr,
                                    const int64_t* offsets, int64_t length, int64_t batch, void* sig,
                                    int64_t sig_stride, const void* seed, int64_t seed_stride, void* grad) {
    return with_plan(plan, dtype, batch, [&]() -> int {
        auto s = static_cast<cudaStream_t>(stream);
        const int threads = scheduled_threads(schedule_key(plan, dtype, true, sig, seed, offsets));
        rpp_gb::PathBatch paths{offsets, length, batch};
        rpp_gb::StaticScratchRefusal refusal = rpp_gb::StaticScratchRefusal::None;
        cudaError_t err;
        if (dtype == RPP_GB_F64) {
            if (int rc = check_signature_args<double>(plan, incr, offsets, length, sig, sig_stride, seed, seed_stride,
                                                      grad, true))
                return rc;
            err = rpp_gb::launch_signature_static_scratch<double>(
                plan->geometry, plan->device, s, static_cast<const double*>(incr), paths, static_cast<double*>(sig),
                sig_stride, static_cast<const double*>(seed), seed_stride, static_cast<double*>(grad), threads,
                &refusal);
        } else {
            if (int rc = check_signature_args<float>(plan, incr, offsets, length, sig, sig_stride, seed, seed_stride,
                                                     grad, true))
                return rc;
            err = rpp_gb::launch_signature_static_scratch<float>(
                plan->geometry, plan->device, s, static_cast<const float*>(incr), paths, static_cast<float*>(sig),
                sig_stride, static_cast<const float*>(seed), seed_stride, static_cast<float*>(grad), threads,
                &refusal);
        }
        if (refusal == rpp_gb::StaticScratchRefusal::BatchTooLarge)
            return fail(RPP_GB_OUT_OF_BOUNDS, "ragged batch of " + std::to_string(batch) +
                                                  " paths exceeds the static scratch capacity of " +
                                                  std::to_string(rpp_gb::static_scratch_max_paths()) + " paths");
        if (refusal == rpp_gb::StaticScratchRefusal::StateTooLarge)
            return fail(RPP_GB_NOT_IMPLEMENTED,
                        "signature state does not fit shared memory; this shape needs the global workspace of "
                        "rpp_gb_signature");
        return cuda_status(err, "signature kernel (static scratch)");
    });
}

int rpp_gb_signature_group(rpp_gb_stream stream, const rpp_gb_signature_job* jobs, int32_t njobs,
                           int32_t schedule) {
    if (!jobs || njobs < 1 || njobs > rpp_gb::kMaxGroupJobs)
        return fail(RPP_GB_INVALID_ARGUMENT, "njobs must be in [1, " + std::to_string(rpp_gb::kMaxGroupJobs) + "]");
    if (schedule < 0 || (schedule & 1023) % 32 != 0 || (schedule & 1023) > 640)
        return fail(RPP_GB_INVALID_ARGUMENT, "schedule: threads per CTA must be a multiple of 32, at most 640");
    rpp_gb::SignatureJob in[rpp_gb::kMaxGroupJobs];
    int device = -1;
    const int cta = (schedule & 1023) ? (schedule & 1023) : 640;
    for (int32_t j = 0; j < njobs; ++j) {
        const rpp_gb_signature_job& job = jobs[j];
        const std::string which = "job " + std::to_string(j) + ": ";
        if (!job.plan) return fail(RPP_GB_INVALID_ARGUMENT, which + "plan is NULL");
        if (!valid_dtype(job.dtype)) return fail(RPP_GB_INVALID_ARGUMENT, which + "unknown dtype");
        if (job.batch < 0) return fail(RPP_GB_INVALID_ARGUMENT, which + "negative batch size");
        if (device < 0) device = job.plan->device.device;
        if (job.plan->device.device != device)
            return fail(RPP_GB_INVALID_ARGUMENT, which + "plans of one group must share a device");
        const int rc = job.dtype == RPP_GB_F64
                           ? check_signature_args<double>(job.plan, job.incr, job.offsets, job.length, job.sig,
                                                          job.sig_stride, job.seed, job.seed_stride, job.grad, true)
                           : check_signature_args<float>(job.plan, job.incr, job.offsets, job.length, job.sig,
                                                         job.sig_stride, job.seed, job.seed_stride, job.grad, true);
        if (rc) return fail(rc, which + rpp_gb_last_error_string());
        const auto& g = job.plan->geometry;
        // threads per team in bits 0-9; bit 26 (kScheduleCotangentGlobal):
        // an FP64 forward + reverse job keeps its cotangent arrays in a global
        // workspace (as the schedule bit of rpp_gb_signature does)
        int t = job.threads & 1023;
        bool cot = (job.threads & rpp_gb::kScheduleCotangentGlobal) != 0;
        if (job.threads < 0 || (job.threads & ~(1023 | rpp_gb::kScheduleCotangentGlobal)) != 0)
            return fail(RPP_GB_INVALID_ARGUMENT, which + "threads: a team size in bits 0-9, optionally bit 26");
        // FP32 jobs of an instantiated shape: one warp per first letter (the
        // kernels of rpp_gb_signature's schedule bit 16: forward-only, and
        // forward + reverse for depth >= 3), unless the caller asks for a
        // team size
        const bool letters = t == 0 && job.dtype == RPP_GB_F32 && 32 * g.width <= cta &&
                             ((job.sig && !job.seed && rpp_gb::letter_warps_supported(g.width, g.depth)) ||
                              (job.seed && rpp_gb::letter_reverse_supported(g.width, g.depth)));
        if (letters) t = 32 * g.width;
        if (t == 0) {
            // the recorded schedule's (forward) CTA size and cotangent
            // workspace, else the heuristic
            const int rec = scheduled_threads(schedule_key(job.plan, job.dtype, true, job.sig, job.seed, job.offsets));
            t = rec & 1023;
            if (!(rec & rpp_gb::kScheduleSplit) && ((rec >> rpp_gb::kScheduleClusterShift) & 7) == 0)
                cot = cot || (rec & rpp_gb::kScheduleCotangentGlobal) != 0;
            if (t == 0)
                for (t = 32; t < 256 && static_cast<uint32_t>(t) < g.pw[g.depth];) t *= 2;
            t = std::max(t, (g.depth * g.width + 31) / 32 * 32);
            t = std::min(t, cta);
        }
        if (t < 32 || t % 32 != 0 || t < g.depth * g.width || t > cta)
            return fail(RPP_GB_INVALID_ARGUMENT,
                        which + "threads must be a multiple of 32, at least width*depth and at most the CTA size");
        in[j] = rpp_gb::SignatureJob{g, job.dtype == RPP_GB_F64, t, letters, job.incr,
                                     rpp_gb::PathBatch{job.offsets, job.length, job.batch}, job.sig, job.sig_stride,
                                     job.seed, job.seed_stride, job.grad};
        in[j].cot = cot && job.dtype == RPP_GB_F64 && job.seed && job.grad;
    }
    DeviceGuard guard(device);
    if (guard.error() != cudaSuccess) return cuda_status(guard.error(), "cudaSetDevice");
    rpp_gb::GroupRefusal refusal = rpp_gb::GroupRefusal::None;
    const cudaError_t err = rpp_gb::launch_signature_group(jobs[0].plan->device, static_cast<cudaStream_t>(stream),
                                                           in, njobs, schedule, &refusal);
    if (refusal == rpp_gb::GroupRefusal::StateTooLarge)
        return fail(RPP_GB_NOT_IMPLEMENTED,
                    "a job's state does not fit one team's shared memory; run it with rpp_gb_signature");
    if (refusal == rpp_gb::GroupRefusal::TooManyPaths)
        return fail(RPP_GB_OUT_OF_BOUNDS, "a job holds at most 2^31 - 1 paths");
    return cuda_status(err, "grouped signature kernel");
}

int rpp_gb_signature_tune(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const void* incr,
                          const int64_t* offsets, int64_t length, int64_t batch, void* sig, int64_t sig_stride,
                          const void* seed, int64_t seed_stride, void* grad, int32_t* threads, float* ms) {
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? tune_signature<double>(plan, s, dtype, incr, offsets, length, batch, sig,
                                                            sig_stride, seed, seed_stride, grad, threads, ms)
                                   : tune_signature<float>(plan, s, dtype, incr, offsets, length, batch, sig,
                                                           sig_stride, seed, seed_stride, grad, threads, ms);
    });
}

int rpp_gb_signature_with_schedule(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype, const void* incr,
                                   const int64_t* offsets, int64_t length, int64_t batch, void* sig,
                                   int64_t sig_stride, const void* seed, int64_t seed_stride, void* grad,
                                   int32_t schedule) {
    if (schedule <= 0) return fail(RPP_GB_INVALID_ARGUMENT, "schedule must be positive");
    return with_plan(plan, dtype, batch, [&] {
        auto s = static_cast<cudaStream_t>(stream);
        return dtype == RPP_GB_F64 ? run_signature<double>(plan, s, dtype, incr, offsets, length, batch, sig,
                                                           sig_stride, seed, seed_stride, grad, true, schedule)
                                   : run_signature<float>(plan, s, dtype, incr, offsets, length, batch, sig,
                                                          sig_stride, seed, seed_stride, grad, true, schedule);
    });
}

}  // extern "C"
