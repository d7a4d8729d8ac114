// signature.cu -- the fused signature kernel (k_signature) and its launches:
// one persistent launch per call (or a forward and a reverse launch, as the
// schedule says), ragged batches ordered longest first, the large-state and
// cotangent-workspace variants, and the allocation-free entry point.  The
// per-path device code and the algorithm it implements are in
// signature_body.cuh.
#include <mutex>

#include "signature_body.cuh"

namespace rpp_gb {
namespace {

// The signature kernel: persistent CTAs, one path at a time (grid-stride over
// the batch, or taken from the ragged batch's work counter).
// Registers: at most 64 per thread for FP64 (two 512-thread blocks per SM;
// the fastest measured), 40 for FP32, whose small states fit more CTAs per SM
// than 64 registers allow (ragged W8 D4 FP32: 29.3 -> 28.3 ms).
// COT: the cotangent arrays may live in the global workspace (kCotGlobal) --
// a separate instantiation, so that the other kernels' code is what it was
// without that option (it cost W16 D3 2.6 % when it was a run-time choice).
// TOPREGS: forward-only FP32 with the top level in registers (kTopRegs), at
// up to 64 registers per thread (32 of them the rows of the top level).
template <typename T, int WT, int MAXT, bool COT = false, bool TOPREGS = false>
__global__ void __launch_bounds__(MAXT, (MAXT <= 512 ? (sizeof(T) == 4 && !TOPREGS ? 3 : 2) : 1)) k_signature(SigGeometry sg, const T* __restrict__ incr, PathBatch paths,
                                                    T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                                                    T* grad, int mode, T* gws, int64_t gws_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const CtaTeam tm;
    bool vec4 = false;
    SigShared<T> sh = place_arrays<T, WT, COT>(tm, sg, mode, gws, gws_stride, smem_raw, vec4);

    __shared__ int64_t s_next;
    int64_t slot = blockIdx.x;
    if (paths.counter) {
        if (threadIdx.x == 0) s_next = static_cast<int64_t>(atomicAdd(paths.counter, 1u));
        __syncthreads();
        slot = s_next;
        __syncthreads();
    }
    for (; slot < paths.batch;) {
        const int64_t b = paths.order ? paths.order[slot] : slot;
        const int64_t off = paths.offsets ? paths.offsets[b] : b * paths.length;
        const int64_t len = paths.offsets ? paths.offsets[b + 1] - off : paths.length;
        run_path<T, WT, TOPREGS>(tm, sg, sh, incr, b, off, len, sig, sig_stride, seed, seed_stride, grad, mode, vec4);
        if (paths.counter) {
            if (threadIdx.x == 0) s_next = static_cast<int64_t>(atomicAdd(paths.counter, 1u));
            __syncthreads();
            slot = s_next;
            __syncthreads();
        } else {
            slot += gridDim.x;
        }
    }
}

// Orders the paths of a ragged batch longest first for the work counter: a
// one-CTA counting sort on a log-scale length key (4 buckets per octave), so
// paths of similar length share a bucket.  The order inside a bucket does not
// matter: every path's result is independent of when it is processed.  Also
// zeroes the counter.
__global__ void __launch_bounds__(1024) k_order_by_length(const int64_t* offsets, int64_t batch, int32_t* order,
                                                          unsigned int* counter) {
    __shared__ unsigned int hist[kLengthBuckets];
    __shared__ unsigned int start[kLengthBuckets];
    for (int i = threadIdx.x; i < kLengthBuckets; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (int64_t b = threadIdx.x; b < batch; b += blockDim.x)
        atomicAdd(&hist[length_bucket(offsets[b + 1] - offsets[b])], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int acc = 0;
        for (int k = kLengthBuckets - 1; k >= 0; --k) {  // longest bucket first
            start[k] = acc;
            acc += hist[k];
        }
        *counter = 0;
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b < batch; b += blockDim.x) {
        const unsigned int pos = atomicAdd(&start[length_bucket(offsets[b + 1] - offsets[b])], 1u);
        order[pos] = static_cast<int32_t>(b);
    }
}


// Pad a CTA's dynamic shared memory so that at most `cap` CTAs fit on an SM
// (fewer, longer waves: 4096 paths over 3 CTAs x 152 SMs is 8.98 waves, over
// 4 x 152 it is 6.74 and the last wave runs a quarter empty).  Returns false
// when the cap would not lower the residency.
template <auto kernel>
bool cap_residency(const DeviceInfo& dev, int threads, int cap, size_t& smem) {
    int natural = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&natural, kernel, threads, smem) != cudaSuccess) return false;
    if (natural <= cap) return false;
    int per_sm = 0, reserved = 0;
    cudaFuncAttributes attr{};
    if (cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev.device) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev.device) != cudaSuccess ||
        cudaFuncGetAttributes(&attr, kernel) != cudaSuccess)
        return false;
    const size_t padded = static_cast<size_t>(per_sm / cap - reserved) - attr.sharedSizeBytes;
    if (padded < smem || padded + attr.sharedSizeBytes > static_cast<size_t>(dev.max_smem_optin)) return false;
    smem = padded;
    return true;
}

// How a launch runs: the shared-memory kernel (Resident), the same kernel
// with its cotangent arrays in a stream-ordered global workspace
// (CotangentWorkspace), or the global-workspace kernel for states larger than
// one CTA's shared memory (Workspace).  Only Resident allocates nothing.
enum class SigVariant { Invalid, Resident, CotangentWorkspace, Workspace };

// The variant launch_width takes for `mode` under `schedule` (CTA size in the
// low 10 bits, 0: heuristic; the cap bits are applied by the caller), with the
// CTA size and dynamic shared memory of the shared-memory variants.  `mode`
// may gain kTopGlobal (a state that misses shared memory by less than its top
// level) and kCotGlobal.
template <typename T>
SigVariant choose_variant(const SigGeometry& sg, const DeviceInfo& dev, int& mode, int schedule, int& threads,
                          size_t& smem) {
    const bool bwd = mode & kBackward;
    const int threads_req = schedule > 0 ? (schedule & 1023) : 0;
    threads = threads_req > 0 ? threads_req : threads_for(sg.g.pw[sg.g.depth]);
    if (threads % 32 != 0 || threads > kResidentMaxThreads) return SigVariant::Invalid;
    smem = sig_smem_bytes<T>(sg, threads, bwd, true, mode & kTopGlobal);
    // (the kernel also holds a few bytes of static shared memory)
    const size_t optin = static_cast<size_t>(dev.max_smem_optin);
    if (smem + 64 > optin && sig_smem_bytes<T>(sg, threads, bwd, true, true) + 64 <= optin) {
        mode |= kTopGlobal;
        smem = sig_smem_bytes<T>(sg, threads, bwd, true, true);
    }
    if (bwd && (schedule & kScheduleCotangentGlobal)) {
        mode |= kCotGlobal;
        smem = sig_smem_bytes<T>(sg, threads, false, true, mode & kTopGlobal);
        if (smem + 64 > optin && !(mode & kTopGlobal)) {  // the top level to global memory too
            mode |= kTopGlobal;
            smem = sig_smem_bytes<T>(sg, threads, false, true, true);
        }
        return smem + 64 > optin ? SigVariant::Invalid : SigVariant::CotangentWorkspace;
    }
    return smem + 64 <= optin ? SigVariant::Resident : SigVariant::Workspace;
}

// `schedule` = CTA size in the low 10 bits (0: heuristic) and an optional cap
// on CTAs per SM above them (0: as many as fit).
template <typename T, int WT>
cudaError_t launch_width(const SigGeometry& sg, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                         PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride, T* grad,
                         int mode, int schedule) {
    const bool bwd = mode & kBackward;
    if constexpr (std::is_same<T, float>::value) {
        // FP32 with one warp per first letter (signature_fp32.cu)
        if (schedule > 0 && (schedule & kScheduleLetterWarps) && !(schedule & kScheduleSplit)) {
            if (mode == (kForward | kTopLevel))
                return launch_signature_letters(sg.g, dev, s, incr, paths, sig, sig_stride);
            if (bwd && letter_reverse_supported(sg.g.width, sg.g.depth))
                return launch_signature_letters_rev(sg.g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride,
                                                    grad, mode);
        }
    }
    const int cluster = schedule > 0 ? ((schedule >> kScheduleClusterShift) & 7) + 1 : 1;
    if (cluster >= 2) {  // the state split over a cluster of CTAs (signature_split.cu)
        // kScheduleForwardTopGlobal: the top level in the signature / seed
        // rows (less shared memory per CTA, more clusters resident)
        const int t = (schedule & 1023) ? (schedule & 1023) : threads_for(sg.g.pw[sg.g.depth] / cluster);
        // kScheduleCotangentGlobal: the cotangent level and chains in a
        // per-CTA global workspace (less shared memory per CTA again)
        int m = (schedule & kScheduleForwardTopGlobal) ? (mode | kTopGlobal) : mode;
        if (bwd && (schedule & kScheduleCotangentGlobal)) m |= kCotGlobal;
        return launch_signature_split<T>(sg.g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, m,
                                         std::max(t, (sg.g.depth * sg.g.width + 31) / 32 * 32), cluster);
    }
    const int cap = schedule > 0 ? ((schedule >> 10) & 15) : 0;
    if (bwd && schedule > 0 && (schedule & kScheduleMergedReverse)) mode |= kMergedReverse;
    int threads = 0;
    size_t smem = 0;
    const SigVariant variant = choose_variant<T>(sg, dev, mode, schedule, threads, smem);
    if (variant == SigVariant::Invalid) return cudaErrorInvalidConfiguration;
    if (variant == SigVariant::CotangentWorkspace) {
        // cotangent level and chains in a stream-ordered global workspace (one
        // slice per CTA, L2-resident: 30 MB for two CTAs per SM at W2 D12
        // FP64), state and forward chains resident: at W2 D12 FP64 the reverse
        // launch drops from 196 KB to 98 KB of shared memory per CTA, two CTAs
        // fit per SM, and fwd+bwd runs 49 079 -> 63 370 paths/s (with a
        // 512-thread reverse launch); at W5 D5 it is slower (105 748 -> 103 799)
        const size_t hsmem = smem;
        constexpr auto kernel = k_signature<T, WT, kResidentMaxThreads, true>;
        cudaError_t err = allow_large_smem<kernel>(dev);
        if (err != cudaSuccess) return err;
        if (threads < sg.g.depth * sg.g.width || threads < sg.g.width) return cudaErrorInvalidConfiguration;
        dim3 grid;
        if ((err = batch_grid(kernel, dev, threads, hsmem, paths.batch, grid)) != cudaSuccess) return err;
        const int64_t stride = static_cast<int64_t>((sg.g.db[sg.g.depth] + sg.chain_total + 31) / 32 * 32);
        T* ws = nullptr;
        err = cudaMallocAsync(reinterpret_cast<void**>(&ws), static_cast<size_t>(grid.x) * stride * sizeof(T), s);
        if (err != cudaSuccess) return err;
        kernel<<<grid, threads, hsmem, s>>>(sg, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, ws, stride);
        err = cudaGetLastError();
        cudaError_t ferr = cudaFreeAsync(ws, s);
        return err != cudaSuccess ? err : ferr;
    }
    if constexpr (kTopRows<T, WT> > 0) {
        // forward-only FP32 (W a multiple of 4) with the top level on chip:
        // the top level's rows in registers (kTopRegs) when they fit
        const int D = sg.g.depth;
        const uint32_t rows = D >= 2 ? sg.g.pw[D - 1] : 0u;
        if (variant == SigVariant::Resident && mode == (kForward | kTopLevel) && D >= 2 &&
            rows <= static_cast<uint32_t>(kTopRows<T, WT> * threads)) {
            constexpr auto kernel = k_signature<T, WT, kResidentMaxThreads, false, true>;
            cudaError_t err = allow_large_smem<kernel>(dev);
            if (err != cudaSuccess) return err;
            if (threads < sg.g.depth * sg.g.width || threads < sg.g.width) return cudaErrorInvalidConfiguration;
            size_t rsmem = sig_smem_bytes<T>(sg, threads, false, true, true);
            if (cap > 0 && !cap_residency<kernel>(dev, threads, cap, rsmem)) return cudaErrorInvalidConfiguration;
            dim3 grid;
            if ((err = batch_grid(kernel, dev, threads, rsmem, paths.batch, grid)) != cudaSuccess) return err;
            kernel<<<grid, threads, rsmem, s>>>(sg, incr, paths, sig, sig_stride, seed, seed_stride, grad,
                                                mode | kTopRegs, nullptr, 0);
            return cudaGetLastError();
        }
    }
    if (variant == SigVariant::Resident) {
        constexpr auto kernel = k_signature<T, WT, kResidentMaxThreads>;
        cudaError_t err = allow_large_smem<kernel>(dev);
        if (err != cudaSuccess) return err;
        // every (degree, letter) pair of the scaled increment needs its own thread
        if (threads < sg.g.depth * sg.g.width || threads < sg.g.width) return cudaErrorInvalidConfiguration;
        if (cap > 0 && !cap_residency<kernel>(dev, threads, cap, smem)) return cudaErrorInvalidConfiguration;
        dim3 grid;
        if ((err = batch_grid(kernel, dev, threads, smem, paths.batch, grid)) != cudaSuccess) return err;
        kernel<<<grid, threads, smem, s>>>(sg, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, nullptr, 0);
        return cudaGetLastError();
    }
    // State larger than one CTA's shared memory: stream-ordered workspace,
    // released on the same stream after the launch, one CTA of kWideThreads
    // per SM -- or, when the workspace of two CTAs per SM still fits well
    // inside L2 (the reverse launch of a two-launch schedule holds no top
    // level: 328 KB per CTA at W6 D6 FP64, 100 MB for 304 CTAs), two CTAs of
    // half the size per SM, whose barriers the SM then overlaps (W6 D6 L128,
    // 512 paths: 10 801 -> 11 035 paths/s).
    if (cap > 0) return cudaErrorInvalidConfiguration;  // one CTA per SM already
    constexpr auto kernel = k_signature<T, 0, kWideThreads>;
    const int64_t stride = static_cast<int64_t>((sig_state_elems(sg, bwd, mode & kTopGlobal) + 31) / 32 * 32);
    const bool two = (mode & kTopGlobal) && 2 * dev.sm_count * stride * sizeof(T) <= (size_t(112) << 20);
    threads = two ? kWideThreads / 2 : kWideThreads;
    if (threads < sg.g.depth * sg.g.width) return cudaErrorInvalidConfiguration;
    smem = sig_smem_bytes<T>(sg, threads, bwd, false);
    const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>(paths.batch, (two ? 2 : 1) * dev.sm_count));
    T* ws = nullptr;
    cudaError_t err = cudaMallocAsync(reinterpret_cast<void**>(&ws), static_cast<size_t>(ctas * stride) * sizeof(T), s);
    if (err != cudaSuccess) return err;
    kernel<<<dim3(static_cast<unsigned>(ctas)), threads, smem, s>>>(sg, incr, paths, sig, sig_stride, seed,
                                                                    seed_stride, grad, mode, ws, stride);
    err = cudaGetLastError();
    cudaError_t ferr = cudaFreeAsync(ws, s);
    return err != cudaSuccess ? err : ferr;
}

template <typename T>
cudaError_t launch_width_any(const SigGeometry& sg, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                             PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride, T* grad,
                             int mode, int threads) {
    switch (sg.g.width) {
        case 2: return launch_width<T, 2>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
        case 3: return launch_width<T, 3>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
        case 4: return launch_width<T, 4>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
        case 5: return launch_width<T, 5>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
        case 6: return launch_width<T, 6>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
        case 8: return launch_width<T, 8>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
        case 16: return launch_width<T, 16>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
        default: return launch_width<T, 0>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads);
    }
}

// The launches of one call: one fused launch, or -- kScheduleSplit, a
// forward+reverse call with signature output -- a forward launch and a
// reverse launch from the final signatures; the reverse launch reads the
// seed's top level from global memory, so both hold less shared memory per
// CTA (more CTAs per SM) than the fused one.
struct SigLaunches {
    int count = 0;
    int mode[2] = {0, 0};
    int schedule[2] = {0, 0};
};

// `letters`: the call is FP32 of a shape the warp-per-letter forward kernel
// is instantiated for; its forward-only launches then take that kernel (bit
// 16 of their own schedule word) unless a schedule fixes the CTA size: the
// forward launch of the two-launch form, and forward-only calls without a
// recorded schedule.  Its results equal the shared-memory kernel's bit for bit.
// `letters_rev`: the shape has the warp-per-letter reverse kernel too, which
// calls with a reverse pass and no recorded schedule then take.
SigLaunches plan_launches(bool forward, bool has_sig, bool has_seed, bool has_grad, int threads,
                          bool letters = false, bool letters_rev = false) {
    SigLaunches l;
    const bool split = forward && has_sig && has_seed && has_grad && threads > 0 && (threads & kScheduleSplit);
    if (split) {
        const bool fwd_top_global = threads & kScheduleForwardTopGlobal;
        const int rev = (threads >> kScheduleReverseShift) & 1023;
        const int cot = threads & (kScheduleCotangentGlobal | kScheduleMergedReverse);
        const int fwd = threads & ((1 << 14) - 1);  // CTA size and cap
        l.count = 2;
        l.mode[0] = kForward | kTopLevel | (fwd_top_global ? kTopGlobal : 0);
        l.schedule[0] = (letters && !fwd_top_global) ? (32 | kScheduleLetterWarps) : fwd;
        l.mode[1] = kBackward | kLoadFinal | kTopGlobal;
        l.schedule[1] = (rev > 0 ? (fwd & ~1023) | rev : fwd) | cot;
        return l;
    }
    int mode = 0;
    if (forward) {
        mode |= kForward;
        if (has_seed && has_grad) mode |= kBackward;
        // The top level of S is only an output: a gradient-only call skips it.
        if (has_sig) mode |= kTopLevel;
    } else {
        mode |= kBackward | kLoadFinal;
    }
    // a forward-only call with kScheduleForwardTopGlobal keeps the top level
    // in the output row (the two-launch form's forward launch does the same)
    if (threads > 0 && (threads & kScheduleForwardTopGlobal) && mode == (kForward | kTopLevel) &&
        ((threads >> kScheduleClusterShift) & 7) == 0)
        mode |= kTopGlobal;
    l.count = 1;
    l.mode[0] = mode;
    const bool letter_kernel = threads == 0 && ((letters && mode == (kForward | kTopLevel)) ||
                                                (letters_rev && (mode & kBackward)));
    l.schedule[0] = letter_kernel ? (32 | kScheduleLetterWarps) : threads;
    return l;
}

// Runs the launches; a ragged batch's work counter is re-armed between them.
template <typename T>
cudaError_t run_launches(const SigGeometry& sg, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                         PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride, T* grad,
                         const SigLaunches& l) {
    cudaError_t err = cudaSuccess;
    for (int i = 0; i < l.count && err == cudaSuccess; ++i) {
        if (i > 0 && paths.counter) err = cudaMemsetAsync(paths.counter, 0, sizeof(unsigned int), s);
        if (err == cudaSuccess)
            err = launch_width_any<T>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, l.mode[i],
                                      l.schedule[i]);
    }
    return err;
}

}  // namespace

template <typename T>
cudaError_t launch_signature(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                             PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                             T* grad, bool forward, int threads) {
    if (paths.batch <= 0) return cudaSuccess;
    const SigGeometry sg = make_sig_geometry(g);
    constexpr bool fp32 = std::is_same<T, float>::value;
    const SigLaunches launches = plan_launches(forward, sig != nullptr, seed != nullptr, grad != nullptr, threads,
                                               fp32 && letter_warps_supported(g.width, g.depth),
                                               fp32 && letter_reverse_supported(g.width, g.depth));
    // Ragged batches: order the paths longest first and hand them out through
    // a work counter (stream-ordered scratch, released after the launch).
    void* scratch = nullptr;
    if (paths.offsets && paths.batch > 1) {
        const size_t bytes = 256 + static_cast<size_t>(paths.batch) * sizeof(int32_t);
        cudaError_t err = cudaMallocAsync(&scratch, bytes, s);
        if (err != cudaSuccess) return err;
        paths.counter = static_cast<unsigned int*>(scratch);
        paths.order = reinterpret_cast<int32_t*>(static_cast<char*>(scratch) + 256);
        k_order_by_length<<<1, 1024, 0, s>>>(paths.offsets, paths.batch, const_cast<int32_t*>(paths.order),
                                             paths.counter);
        if ((err = cudaGetLastError()) != cudaSuccess) {
            cudaFreeAsync(scratch, s);
            return err;
        }
    }
    cudaError_t err = run_launches<T>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, launches);
    if (scratch) {
        cudaError_t ferr = cudaFreeAsync(scratch, s);
        if (err == cudaSuccess) err = ferr;
    }
    return err;
}

// ---------------------------------------------------------------------------
// Allocation-free variant (rpp_gb_signature_static_scratch).
//
// Some callers cannot allocate device memory at call time: runtimes that own
// the whole device memory through their own allocator (and forbid raw
// cudaMalloc / cudaMallocAsync from plugins), real-time loops that must not
// wait on or grow a memory pool, and hosts that budget device memory up front.
// For them the ragged-batch scratch (the work counter and the longest-first
// path order) lives in this fixed, file-scope device array instead of a
// stream-ordered allocation.  Every GPU that loads the library holds the
// array (8 MiB) until the process exits.  All calls share it and it keeps the
// previous call's contents: the ordering kernel rewrites the order and zeroes
// the counter on every call, and calls whose launches overlap on the GPU (on
// different streams, or on one device from several threads without ordering)
// race on it, so such calls must be serialised by the caller.  Host code only
// holds a stand-in for the array's name; its device address is obtained once
// per device, with that device current, by cudaGetSymbolAddress on the first
// call made on that device (so that first call should come before any stream
// capture) and kept for the life of the process: like the plans, whose device
// tables live in the same context, it assumes the device's context is not
// destroyed (cudaDeviceReset) while the library is in use.
namespace {

constexpr size_t kStaticScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_signature_scratch[kStaticScratchBytes];

std::mutex g_scratch_lock;
void* g_scratch_address[kMaxDevices] = {};

cudaError_t static_scratch_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> guard(g_scratch_lock);
    if (!g_scratch_address[device]) {
        void* ptr = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&ptr, g_signature_scratch);
        if (err != cudaSuccess) return err;
        g_scratch_address[device] = ptr;
    }
    *out = g_scratch_address[device];
    return cudaSuccess;
}

}  // namespace

int64_t static_scratch_max_paths() { return static_cast<int64_t>((kStaticScratchBytes - 256) / sizeof(int32_t)); }

template <typename T>
cudaError_t launch_signature_static_scratch(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                                            PathBatch paths, T* sig, int64_t sig_stride, const T* seed,
                                            int64_t seed_stride, T* grad, int threads, StaticScratchRefusal* refusal) {
    *refusal = StaticScratchRefusal::None;
    if (paths.batch <= 0) return cudaSuccess;
    const SigGeometry sg = make_sig_geometry(g);
    // A recorded schedule is honoured except for its cotangent workspace,
    // which is an allocation: that launch runs with its cotangent arrays in
    // shared memory instead (same results).
    if (threads > 0) threads &= ~kScheduleCotangentGlobal;
    constexpr bool fp32 = std::is_same<T, float>::value;
    const SigLaunches launches = plan_launches(true, sig != nullptr, seed != nullptr, grad != nullptr, threads,
                                               fp32 && letter_warps_supported(g.width, g.depth),
                                               fp32 && letter_reverse_supported(g.width, g.depth));
    // Only the shared-memory kernel allocates nothing: every launch of the
    // call must take it, checked before anything is launched.
    for (int i = 0; i < launches.count; ++i) {
        int mode = launches.mode[i], t = 0;
        size_t smem = 0;
        const SigVariant v = choose_variant<T>(sg, dev, mode, launches.schedule[i], t, smem);
        if (v == SigVariant::Workspace || v == SigVariant::CotangentWorkspace) {
            *refusal = StaticScratchRefusal::StateTooLarge;
            return cudaErrorNotSupported;
        }
        if (v == SigVariant::Invalid) return cudaErrorInvalidConfiguration;
    }
    if (paths.offsets && paths.batch > 1) {
        if (paths.batch > static_scratch_max_paths()) {
            *refusal = StaticScratchRefusal::BatchTooLarge;
            return cudaErrorNotSupported;
        }
        void* base = nullptr;
        cudaError_t err = static_scratch_address(dev.device, &base);
        if (err != cudaSuccess) return err;
        paths.counter = static_cast<unsigned int*>(base);
        paths.order = reinterpret_cast<int32_t*>(static_cast<char*>(base) + 256);
        // rewrites the order and zeroes the counter: nothing of the previous
        // call's contents is read
        k_order_by_length<<<1, 1024, 0, s>>>(paths.offsets, paths.batch, const_cast<int32_t*>(paths.order),
                                             paths.counter);
        if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    return run_launches<T>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, launches);
}

template cudaError_t launch_signature_static_scratch<float>(const Geometry&, const DeviceInfo&, cudaStream_t,
                                                            const float*, PathBatch, float*, int64_t, const float*,
                                                            int64_t, float*, int, StaticScratchRefusal*);
template cudaError_t launch_signature_static_scratch<double>(const Geometry&, const DeviceInfo&, cudaStream_t,
                                                             const double*, PathBatch, double*, int64_t,
                                                             const double*, int64_t, double*, int,
                                                             StaticScratchRefusal*);

template cudaError_t launch_signature<float>(const Geometry&, const DeviceInfo&, cudaStream_t, const float*,
                                             PathBatch, float*, int64_t, const float*, int64_t, float*, bool, int);
template cudaError_t launch_signature<double>(const Geometry&, const DeviceInfo&, cudaStream_t, const double*,
                                              PathBatch, double*, int64_t, const double*, int64_t, double*, bool,
                                              int);

}  // namespace rpp_gb
