// ops.hpp -- host-side launchers of the sm_103a kernels (internal; the public
// surface is the C ABI in include/rpp_gb300.h).  Every launcher enqueues on
// `stream` and returns the launch's cudaError_t.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace rpp_gb {

enum class ProductKind : int {
    Fma = 0,         // out = alpha*a + beta*b(x)c   (a may be absent)
    InplaceBCA = 1,  // a = alpha*a + beta*b(x)c
    InplaceABC = 2,  // a = alpha*c + beta*a(x)b
    InplaceBAC = 3,  // a = alpha*c + beta*b(x)a
    InplaceMul = 4,  // a = beta*a(x)b
};

enum class IntermediateKind : int { Exp = 0, FMExp = 1, Log = 2 };

enum class HelperKind : int { Assign = 0, SetConstant = 1, SetIdentity = 2, AddIdentity = 3 };

struct DeviceInfo {
    int device;
    int sm_count;
    int max_smem_optin;
};

template <typename T>
cudaError_t launch_product(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, ProductKind kind,
                           TArg<T> out, TArg<T> x, TArg<T> y, TArg<T> z, int64_t batch, double alpha,
                           double beta);

template <typename T>
cudaError_t launch_intermediate(const Geometry& g, const DeviceInfo& dev, cudaStream_t s,
                                IntermediateKind kind, TArg<T> out, TArg<T> x, TArg<T> y,
                                int64_t batch);

template <typename T>
cudaError_t launch_adjoint(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, bool left,
                           TArg<T> out, TArg<T> op, TArg<T> arg, int64_t batch);

template <typename T>
cudaError_t launch_antipode(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, bool sign,
                            TArg<T> out, TArg<T> arg, int64_t batch);

template <typename T>
cudaError_t launch_helper(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, HelperKind kind,
                          TArg<T> out, TArg<T> arg, int64_t batch, double value);

template <typename T>
cudaError_t launch_exp_letter_vjp(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* H,
                                  int64_t h_stride, const T* x, int64_t x_stride, T* dx, int64_t dx_stride,
                                  int64_t batch);

// CSR SpMM over a batch of begin-relative vector views.
struct CsrDevice {
    const int32_t* offsets;  // rows + 1
    const int32_t* cols;     // nnz
    const double* values64;  // nnz
    const float* values32;   // nnz
    int64_t rows;
    int64_t cols_dim;
    int64_t nnz;
    bool zero_rest;  // matrix came from CSC: zero the whole out view first
    uint32_t* fault; // fault word for expired bounded waits (see Geometry::fault)
    // Sliced copy for the SpMM kernels (sliced ELL, 32 rows per slice): the
    // rows in decreasing number of entries (ties in row order) are cut into
    // slices of 32, and entry k of the slice's row l sits at
    // slice_off[s] + 32*k + l.  A warp takes a slice and lane l walks its row:
    // the warp's loads of entry k are one contiguous span, and the rows of a
    // warp have nearly equal lengths, so its FMA instructions run with nearly
    // all lanes active (a warp issues as many as its longest row has entries).
    const int32_t* order;      // rows: the row at sorted position i
    const int32_t* row_len;    // rows: its number of entries
    const int32_t* slice_off;  // slices + 1 (multiples of 32)
    const int32_t* ell_cols;   // slice_off[slices]; padding is never read
    const double* ell_v64;
    const float* ell_v32;
};

template <typename T>
cudaError_t launch_spmm(const CsrDevice& m, const DeviceInfo& dev, cudaStream_t s, T* out,
                        int64_t out_stride, int64_t out_size, const T* arg, int64_t arg_stride,
                        int64_t arg_size, int64_t batch, double alpha);

// Shuffle algebra (shuffle.cu).
enum class ShuffleKind : int {
    Mul = 0,         // out = beta * lhs sh rhs
    Fma = 1,         // out = alpha*add + beta * lhs sh rhs   (add may be absent)
    InplaceFma = 2,  // out = alpha*out + beta * lhs sh rhs
    LeftHalf = 3,    // out = beta * lhs < rhs, out[0] = 0
};

enum class ShuffleAdjKind : int {
    Shuffle = 0,  // st_adj_mul(out, op, arg)
    HalfL = 1,    // left_hs_adj_lmul: op = integrator, arg = integrand
    HalfR = 2,    // left_hs_adj_rmul: op = integrand, arg = integrator
};

// Order in which a shuffle kernel visits the output degrees: entry e covers
// degree deg[e], output positions [start[e], start[e+1]); the first
// warp_entries entries give each coefficient a warp.
struct ShuffleOrder {
    int count;
    int warp_entries;
    int tasked;  // adjoints: entries [tasked, count) have no terms and are zero-filled, not queued
    int deg[kMaxDepth + 1];
    uint32_t start[kMaxDepth + 2];
};

ShuffleOrder shuffle_product_order(const Geometry& g, int out_lo, int out_hi);
ShuffleOrder shuffle_adjoint_order(const Geometry& g, ShuffleAdjKind kind, int out_lo, int out_hi, int op_lo,
                                   int op_hi, int arg_lo, int arg_hi, int threads);

template <typename T>
cudaError_t launch_shuffle_product(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, ShuffleKind kind,
                                   TArg<T> out, TArg<T> add, TArg<T> lhs, TArg<T> rhs, int64_t batch, double alpha,
                                   double beta, const ShuffleOrder& ord);

// `op` is the fixed operand, `arg` the cotangent (the kernels' reading order).
template <typename T>
cudaError_t launch_shuffle_adjoint(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, ShuffleAdjKind kind,
                                   TArg<T> out, TArg<T> op, TArg<T> arg, int64_t batch, double beta);

template <typename T>
cudaError_t launch_pairing(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, T* result, TArg<T> f, TArg<T> a,
                           int64_t batch);

// Fused Lie <-> tensor steps (lie_fused.cu).  Both need their work tensors in
// shared memory: *_smem gives the bytes, the caller composes the unfused
// kernels when it exceeds the device's limit.
size_t log_to_lie_smem(const Geometry& g, size_t elem);
size_t lie_exp_smem(const Geometry& g, size_t elem, bool fm);

// out (begin-relative, out_size coefficients) = alpha * M * log(x)|[lo, hi]
template <typename T>
cudaError_t launch_log_to_lie(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const CsrDevice& m,
                              TArg<T> x, int lo, int hi, T* out, int64_t out_stride, int64_t out_size, int64_t batch,
                              double alpha);

// out = exp(X) or mult (x) exp(X), X = alpha * M * lie on degrees [lo, hi]
template <typename T>
cudaError_t launch_lie_exp(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const CsrDevice& m,
                           const T* lie, int64_t lie_stride, int lo, int hi, TArg<T> out, TArg<T> mult,
                           int64_t batch, double alpha);

// Self-test of the bounded mbarrier wait (peak_probe.cu): one CTA waits,
// with a short limit, for a transaction that nothing completes; the wait
// expires, the fault word gets kFaultBulkWait and the kernel returns.
cudaError_t launch_expired_wait(const Geometry& g, cudaStream_t s);

// Fused signature kernels.
struct PathBatch {
    const int64_t* offsets;  // device, batch + 1 (or nullptr)
    int64_t length;          // equal length when offsets == nullptr
    int64_t batch;
    // Ragged batches: paths are handed out longest first through a work
    // counter (order[] lists path indices by decreasing length, both device
    // scratch written by the launcher).  Null for equal-length batches.
    const int32_t* order = nullptr;
    unsigned int* counter = nullptr;
};

// `threads` = the schedule: CTA size of the shared-memory variant in bits
// 0-9 (0: heuristic), a cap on CTAs per SM in bits 10-13 (0: none), and
// kScheduleSplit: run a forward+reverse call with signature output as a
// forward launch plus a reverse launch from the final signatures;
// kScheduleForwardTopGlobal (with kScheduleSplit, or on a forward-only call):
// the forward launch keeps the top level in the output row in global memory
// (less shared memory per CTA, more CTAs per SM); with kScheduleSplit, bits
// 16-25 (when not 0) give
// the reverse launch its own CTA size (bits 0-9 then size the forward launch).
constexpr int kScheduleSplit = 1 << 14;
constexpr int kScheduleForwardTopGlobal = 1 << 15;
constexpr int kScheduleReverseShift = 16;
// kScheduleCotangentGlobal: a launch with a reverse pass keeps the state and
// the forward chains in shared memory and the cotangent level and chains in
// a per-CTA global workspace (L2-resident), so more CTAs fit per SM.
constexpr int kScheduleCotangentGlobal = 1 << 26;
// kScheduleMergedReverse: reverse steps with D barriers (the recovery of the
// prefix beside the transposition of the cotangent chains) instead of 2D - 1.
constexpr int kScheduleMergedReverse = 1 << 27;
// Bits 28-30 = P - 1: P >= 2 splits each path's state over a cluster of P
// CTAs by first letter (P <= 8 divides the width; one fused launch;
// signature_split.cu);
// with kScheduleForwardTopGlobal the top level then lives in the signature
// and seed rows.
constexpr int kScheduleClusterShift = 28;
template <typename T>
cudaError_t launch_signature(const Geometry& g, const DeviceInfo& dev, cudaStream_t s,
                             const T* incr, PathBatch paths, T* sig, int64_t sig_stride,
                             const T* seed, int64_t seed_stride, T* grad, bool forward, int threads);

// kScheduleLetterWarps (bit 16 of an FP32 call's schedule without
// kScheduleSplit, where bits 16-25 have no other use): the FP32 kernels with
// one warp per first letter and compile-time (width, depth)
// (signature_fp32.cu) -- the forward-only kernel, and for calls with a
// reverse pass (depth >= 3) the forward + reverse kernel.
constexpr int kScheduleLetterWarps = 1 << 16;
bool letter_warps_supported(int width, int depth);
bool letter_reverse_supported(int width, int depth);
cudaError_t launch_signature_letters(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const float* incr,
                                     PathBatch paths, float* sig, int64_t sig_stride);
// `mode`: kForward | kBackward [| kTopLevel], or kBackward | kLoadFinal.
cudaError_t launch_signature_letters_rev(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const float* incr,
                                         PathBatch paths, float* sig, int64_t sig_stride, const float* seed,
                                         int64_t seed_stride, float* grad, int mode);

// Split-state launch (kScheduleClusterShift): `mode` as launch_width's, CTA
// size `threads`, `P` CTAs per cluster.
template <typename T>
cudaError_t launch_signature_split(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                                   PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                                   T* grad, int mode, int threads, int P);

// Grouped signature launch (rpp_gb_signature_group): several jobs -- batches
// of paths of different (width, depth) and precision, each with its own
// inputs and outputs -- in one persistent launch.  Each path of job j is run
// by a team of `threads` threads of a CTA (several teams per CTA when the
// job's state is small), with the per-path code of launch_signature, so its
// outputs equal those of a separate call with that CTA size.
constexpr int kMaxGroupJobs = 8;
struct SignatureJob {
    Geometry g;
    bool fp64;
    int threads;  // team size (a multiple of 32, at least width * depth)
    bool letters;  // FP32: a team of width warps, one per first letter (threads = 32 width; forward-only, or
                   // forward + reverse at depth >= 3)
    const void* incr;
    PathBatch paths;
    void* sig;
    int64_t sig_stride;
    const void* seed;
    int64_t seed_stride;
    void* grad;
    // FP64 forward + reverse: the cotangent level and chains in a per-team
    // slice of a global workspace (kScheduleCotangentGlobal), the state and
    // forward chains in the team's shared memory
    bool cot = false;
};
// Refusal reasons beside the CUDA status.
enum class GroupRefusal : int { None = 0, StateTooLarge = 1, TooManyPaths = 2 };
// `schedule`: threads per CTA in bits 0-9 (at most 640; 0: 640) and
// kScheduleMergedReverse.
cudaError_t launch_signature_group(const DeviceInfo& dev, cudaStream_t s, const SignatureJob* jobs, int njobs,
                                   int schedule, GroupRefusal* refusal);

// Allocation-free signature launch: the ragged-batch scratch lives in a
// fixed device array of the library (see signature.cu); refuses shapes whose
// state needs the global-workspace kernel and batches beyond the array.
enum class StaticScratchRefusal : int { None = 0, StateTooLarge = 1, BatchTooLarge = 2 };

int64_t static_scratch_max_paths();

template <typename T>
cudaError_t launch_signature_static_scratch(const Geometry& g, const DeviceInfo& dev, cudaStream_t s,
                                            const T* incr, PathBatch paths, T* sig, int64_t sig_stride,
                                            const T* seed, int64_t seed_stride, T* grad, int threads,
                                            StaticScratchRefusal* refusal);

}  // namespace rpp_gb
