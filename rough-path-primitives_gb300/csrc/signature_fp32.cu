// signature_fp32.cu -- FP32 signatures with one warp per first letter
// (schedule bit 16, kScheduleLetterWarps): the forward-only kernel, the
// forward + reverse kernel, and their launches; the steps and per-path code
// are in signature_letters.cuh.
#include "signature_letters.cuh"

namespace rpp_gb {
namespace {

// CTAs per SM the register budget is sized for: 32 warps per SM (64
// registers a thread), or 20 (about 100 registers) for the shapes whose
// lower levels and top rows spilled at 64 (W5 D5, W3 D6).
constexpr int letter_min_blocks(int W, int D) {
    return ((W == 5 && D == 5) || (W == 3 && D == 6)) ? 640 / (W * 32) : 1024 / (W * 32);
}

template <int W, int D>
__global__ void __launch_bounds__(W * 32, letter_min_blocks(W, D)) k_signature_letters(const float* __restrict__ incr, PathBatch paths,
                                                              float* sig, int64_t sig_stride) {
    extern __shared__ __align__(16) float sm_letters[];
    __shared__ int64_t s_next;
    const uint32_t c = threadIdx.x / 32;  // this warp's first letter
    const uint32_t lane = threadIdx.x % 32;
    float* region = sm_letters + c * LetterLayout<W, D>::warp_floats;
    int64_t slot = blockIdx.x;
    if (paths.counter) {
        if (threadIdx.x == 0) s_next = static_cast<int64_t>(atomicAdd(paths.counter, 1u));
        __syncthreads();
        slot = s_next;
        __syncthreads();
    }
    while (slot < paths.batch) {
        const int64_t b = paths.order ? paths.order[slot] : slot;
        const int64_t off = paths.offsets ? paths.offsets[b] : b * paths.length;
        const int64_t len = paths.offsets ? paths.offsets[b + 1] - off : paths.length;
        letter_path<W, D>(incr, b, off, len, sig, sig_stride, region, c, lane);
        if (paths.counter) {
            __syncthreads();  // every warp has read s_next
            if (threadIdx.x == 0) s_next = static_cast<int64_t>(atomicAdd(paths.counter, 1u));
            __syncthreads();
            slot = s_next;
        } else {
            slot += gridDim.x;
        }
    }
}

// Registers for the reverse kernel: 20 warps per SM, about 100 registers a
// thread (the seed's top rows, level D-1 and the lane's lower coefficients of
// S and G, the letter sums and the increment ring; at 24 warps per SM, W8 D4
// and W3 D6 spilled).
constexpr int letter_rev_min_blocks(int W) { return 640 / (W * 32) > 0 ? 640 / (W * 32) : 1; }

// Forward + reverse (or reverse from the final signature) with one warp per
// first letter: a CTA of W warps runs one path at a time.
template <int W, int D>
__global__ void __launch_bounds__(W * 32, letter_rev_min_blocks(W))
    k_signature_letters_rev(const float* __restrict__ incr, PathBatch paths, float* sig, int64_t sig_stride,
                            const float* __restrict__ seed, int64_t seed_stride, float* grad, int mode) {
    using Rev = LetterRevLayout<W, D>;
    extern __shared__ __align__(16) float sm_letters[];
    __shared__ int64_t s_next;
    const uint32_t c = threadIdx.x / 32;
    const uint32_t lane = threadIdx.x % 32;
    float* region = sm_letters + c * Rev::warp_floats;
    float* pbuf = sm_letters + W * Rev::warp_floats;
    int64_t slot = blockIdx.x;
    if (paths.counter) {
        if (threadIdx.x == 0) s_next = static_cast<int64_t>(atomicAdd(paths.counter, 1u));
        __syncthreads();
        slot = s_next;
        __syncthreads();
    }
    while (slot < paths.batch) {
        const int64_t b = paths.order ? paths.order[slot] : slot;
        const int64_t off = paths.offsets ? paths.offsets[b] : b * paths.length;
        const int64_t len = paths.offsets ? paths.offsets[b + 1] - off : paths.length;
        letter_fwd_bwd<W, D>(CtaTeam{}, incr, b, off, len, sig, sig_stride, seed, seed_stride, grad, mode, region,
                             pbuf, c, lane);
        __syncthreads();  // the last block's partials are read before the next path writes pbuf
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

template <int W, int D>
cudaError_t launch_letters_rev_shape(const DeviceInfo& dev, cudaStream_t s, const float* incr, PathBatch paths,
                                     float* sig, int64_t sig_stride, const float* seed, int64_t seed_stride,
                                     float* grad, int mode) {
    using Rev = LetterRevLayout<W, D>;
    constexpr auto kernel = k_signature_letters_rev<W, D>;
    const size_t smem = (static_cast<size_t>(W) * Rev::warp_floats + Rev::pbuf_floats) * sizeof(float);
    dim3 grid;
    cudaError_t err = batch_grid(kernel, dev, W * 32, smem, paths.batch, grid);
    if (err != cudaSuccess) return err;
    kernel<<<grid, W * 32, smem, s>>>(incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
    return cudaGetLastError();
}

// The reverse kernel needs level D-1 in registers (D >= 3).
template <int W, int D>
cudaError_t launch_letters_rev_if(const DeviceInfo& dev, cudaStream_t s, const float* incr, PathBatch paths,
                                  float* sig, int64_t sig_stride, const float* seed, int64_t seed_stride, float* grad,
                                  int mode) {
    if constexpr (D >= 3)
        return launch_letters_rev_shape<W, D>(dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
    else
        return cudaErrorInvalidConfiguration;
}

template <int W, int D>
cudaError_t launch_letters_shape(const DeviceInfo& dev, cudaStream_t s, const float* incr, PathBatch paths,
                                 float* sig, int64_t sig_stride) {
    using Lay = LetterLayout<W, D>;
    constexpr auto kernel = k_signature_letters<W, D>;
    const size_t smem = static_cast<size_t>(W) * Lay::warp_floats * sizeof(float);
    dim3 grid;
    cudaError_t err = batch_grid(kernel, dev, W * 32, smem, paths.batch, grid);
    if (err != cudaSuccess) return err;
    kernel<<<grid, W * 32, smem, s>>>(incr, paths, sig, sig_stride);
    return cudaGetLastError();
}

}  // namespace

bool letter_warps_supported(int width, int depth) {
    switch (width * 100 + depth) {
#define RPP_GB_LETTER_CASE(w, d) case w * 100 + d: return true;
        RPP_GB_LETTER_SHAPES(RPP_GB_LETTER_CASE)
#undef RPP_GB_LETTER_CASE
        default: return false;
    }
}

bool letter_reverse_supported(int width, int depth) { return depth >= 3 && letter_warps_supported(width, depth); }

cudaError_t launch_signature_letters_rev(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const float* incr,
                                         PathBatch paths, float* sig, int64_t sig_stride, const float* seed,
                                         int64_t seed_stride, float* grad, int mode) {
    switch (g.width * 100 + g.depth) {
#define RPP_GB_LETTER_CASE(w, d) \
    case w * 100 + d: return launch_letters_rev_if<w, d>(dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        RPP_GB_LETTER_SHAPES(RPP_GB_LETTER_CASE)
#undef RPP_GB_LETTER_CASE
        default: return cudaErrorInvalidConfiguration;
    }
}

cudaError_t launch_signature_letters(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const float* incr,
                                     PathBatch paths, float* sig, int64_t sig_stride) {
    switch (g.width * 100 + g.depth) {
#define RPP_GB_LETTER_CASE(w, d) \
    case w * 100 + d: return launch_letters_shape<w, d>(dev, s, incr, paths, sig, sig_stride);
        RPP_GB_LETTER_SHAPES(RPP_GB_LETTER_CASE)
#undef RPP_GB_LETTER_CASE
        default: return cudaErrorInvalidConfiguration;
    }
}

}  // namespace rpp_gb
