// signature.cu -- fused signature forward / reverse kernels.
//
// One CTA owns one path at a time (grid-stride over the batch) and keeps the
// running signature S in shared memory for all of the path's increments: the
// reference's caller instead launches ft_fmexp once per increment and round-
// trips the whole state through global memory every step
// (tests/rpp/gpu/block/ops/ft_fmexp_tests.cu:126-147).
//
// Chen step, S <- S (x) exp(x) for a degree-one increment x (the case of
// include/rpp/operations/intermediate/ft_fmexp.hpp:66-87 with the exponent
// in degree one): for every level n the Horner chain
//     T^n_0 = S_0,  T^n_j = S_j + T^n_{j-1} (x) x / (n - j + 1),  S_n <- T^n_n
// costs sum_j W^j FMAs, so a step costs F = sum_{i=1..D} (D-i+1) W^i FMAs.
// All chains of one "stage" j are computed together (one barrier per stage)
// from the old levels; the last stage updates every level at once.
//
// Reverse pass for loss = <seed, S_L>: with G = dloss/dS_k, step k needs the
// prefix S_{k-1}.  It is recovered from S_k by running the same chains
// bottom-up: S_j = S'_j - T^j_{j-1} (x) x, then T^n_j = S_j + T^n_{j-1} (x) x c
// (c = 1/(n-j+1)), which also rebuilds every forward chain value (cost F).
// The chains are then transposed top-down:
//     Gbar^n_{T_{j-1}}[u] = c sum_a Gbar^n_{T_j}[ua] x_a        (cost F)
//     xbar_a += c sum_u Gbar^n_{T_j}[ua] T^n_{j-1}[u]             (cost F)
// with Gbar^n_{T_n} = G_n, and G_{k-1} = sum_n Gbar^n_{T_j} per level.  So
// forward + reverse = 4 F per increment, nothing stored per step.
#include "common.cuh"
#include "launch_util.cuh"
#include "ops.hpp"

namespace rpp_gb {
namespace {

// Chain storage: stage j (0 <= j < D) holds the chains n = j+1..D, each W^j
// long, at choff[j] + (n-j-1) W^j.
struct SigGeometry {
    Geometry g;
    uint32_t choff[kMaxDepth + 2];
    uint32_t chain_total;
};

enum SigMode : int { kForward = 1, kBackward = 2, kLoadFinal = 4 };

template <typename T>
struct SigShared {
    T* S;
    T* G;
    T* Tf;
    T* Tb;
    T* xc;    // xc[m*W + a] = x_a / m, m = 1..D
    T* inv;   // inv[m] = 1/m
    T* xbar;  // per-thread partial sums, blockDim.x rows of W
};

template <typename T>
__device__ __forceinline__ const T* chain(const SigGeometry& sg, const T* base, int n, int j) {
    return base + sg.choff[j] + static_cast<uint32_t>(n - j - 1) * sg.g.pw[j];
}
template <typename T>
__device__ __forceinline__ T* chain(const SigGeometry& sg, T* base, int n, int j) {
    return base + sg.choff[j] + static_cast<uint32_t>(n - j - 1) * sg.g.pw[j];
}

// Every thread with t < D*W refreshes one scaled increment coefficient.
template <typename T>
__device__ __forceinline__ void set_increment(const SigGeometry& sg, const SigShared<T>& sh, T xv) {
    const uint32_t W = static_cast<uint32_t>(sg.g.width);
    const uint32_t t = threadIdx.x;
    if (t < static_cast<uint32_t>(sg.g.depth) * W) {
        const uint32_t m = 1 + t / W;
        sh.xc[m * W + t % W] = xv * sh.inv[m];
    }
}

template <typename T>
__device__ __forceinline__ T load_increment(const SigGeometry& sg, const T* path_incr, int64_t k) {
    const uint32_t W = static_cast<uint32_t>(sg.g.width);
    const uint32_t t = threadIdx.x;
    if (t < static_cast<uint32_t>(sg.g.depth) * W) return path_incr[k * W + t % W];
    return T(0);
}

// S <- S (x) exp(x), x given by sh.xc.  Ends with a barrier.
template <typename T>
__device__ void forward_step(const SigGeometry& sg, const SigShared<T>& sh) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    T* S = sh.S;
    const T s0 = S[0];
    for (int j = 1; j < D; ++j) {
        const uint32_t wj = G.pw[j];
        const T* Sj = S + G.db[j];
        for (int n = j + 1; n <= D; ++n) {
            T* dst = chain(sg, sh.Tf, n, j);
            const T* prev = j == 1 ? nullptr : chain(sg, static_cast<const T*>(sh.Tf), n, j - 1);
            const T* xm = sh.xc + (n - j + 1) * W;
            for (uint32_t u = threadIdx.x; u < wj; u += blockDim.x) {
                uint32_t q, a;
                G.divw.divmod(u, q, a);
                const T p = j == 1 ? s0 : prev[q];
                dst[u] = fma(p, xm[a], Sj[u]);
            }
        }
        __syncthreads();
    }
    const T* x1 = sh.xc + W;
    for (int n = 1; n <= D; ++n) {
        const uint32_t wn = G.pw[n];
        T* Sn = S + G.db[n];
        const T* prev = n == 1 ? nullptr : chain(sg, static_cast<const T*>(sh.Tf), n, n - 1);
        for (uint32_t u = threadIdx.x; u < wn; u += blockDim.x) {
            uint32_t q, a;
            G.divw.divmod(u, q, a);
            const T p = n == 1 ? s0 : prev[q];
            Sn[u] = fma(p, x1[a], Sn[u]);
        }
    }
    __syncthreads();
}

// One reverse step: S_k -> S_{k-1} (in place), G_k -> G_{k-1} (in place),
// grad_k <- xbar.  Ends with a barrier.
template <typename T>
__device__ void backward_step(const SigGeometry& sg, const SigShared<T>& sh, T* grad_k) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    T* S = sh.S;
    const T s0 = S[0];
    const T* x1 = sh.xc + W;

    // Phase A: recover S_{k-1} and the forward chains, bottom-up.
    for (int j = 1; j <= D; ++j) {
        const uint32_t wj = G.pw[j];
        T* Sj = S + G.db[j];
        const T* own = j == 1 ? nullptr : chain(sg, static_cast<const T*>(sh.Tf), j, j - 1);
        for (uint32_t u = threadIdx.x; u < wj; u += blockDim.x) {
            uint32_t q, a;
            G.divw.divmod(u, q, a);
            const T s = fma(-(j == 1 ? s0 : own[q]), x1[a], Sj[u]);
            Sj[u] = s;
            for (int n = j + 1; n <= D; ++n) {
                const T p = j == 1 ? s0 : chain(sg, static_cast<const T*>(sh.Tf), n, j - 1)[q];
                chain(sg, sh.Tf, n, j)[u] = fma(p, sh.xc[(n - j + 1) * W + a], s);
            }
        }
        __syncthreads();
    }

    // Phase B: transpose the chains top-down; xbar partials per thread.
    T* xb = sh.xbar + threadIdx.x * W;
    for (uint32_t a = 0; a < W; ++a) xb[a] = T(0);
    for (int j = D; j >= 1; --j) {
        const uint32_t wjm1 = G.pw[j - 1];
        for (int n = j; n <= D; ++n) {
            const int m = n - j + 1;
            const T* gin = n == j ? sh.G + G.db[j] : chain(sg, static_cast<const T*>(sh.Tb), n, j);
            T* gout = chain(sg, sh.Tb, n, j - 1);
            const T* tprev = j == 1 ? nullptr : chain(sg, static_cast<const T*>(sh.Tf), n, j - 1);
            const T* xm = sh.xc + m * W;
            const T c = sh.inv[m];
            for (uint32_t u = threadIdx.x; u < wjm1; u += blockDim.x) {
                const T* grow = gin + u * W;
                const T tt = (j == 1 ? s0 : tprev[u]) * c;
                T acc = T(0);
                for (uint32_t a = 0; a < W; ++a) {
                    const T g = grow[a];
                    acc = fma(g, xm[a], acc);
                    xb[a] = fma(g, tt, xb[a]);
                }
                gout[u] = acc;
            }
        }
        __syncthreads();
    }

    // G_{k-1}: add the chains' contributions to each level below the top.
    for (int j = 0; j < D; ++j) {
        const uint32_t wj = G.pw[j];
        T* Gj = sh.G + G.db[j];
        for (uint32_t u = threadIdx.x; u < wj; u += blockDim.x) {
            T s = Gj[u];
            for (int n = j + 1; n <= D; ++n) s += chain(sg, static_cast<const T*>(sh.Tb), n, j)[u];
            Gj[u] = s;
        }
    }
    // grad_k = sum over threads of the partials (warp w reduces letters w, w+nw, ...).
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (uint32_t a = warp; a < W; a += nwarps) {
        T v = T(0);
        for (uint32_t t = lane; t < blockDim.x; t += 32) v += sh.xbar[t * W + a];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) grad_k[a] = v;
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(256) k_signature(SigGeometry sg, const T* __restrict__ incr,
                                                   PathBatch paths, T* sig, int64_t sig_stride,
                                                   const T* seed, int64_t seed_stride, T* grad,
                                                   int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t dim = G.dim;
    const bool bwd = mode & kBackward;

    SigShared<T> sh;
    T* p = reinterpret_cast<T*>(smem_raw);
    sh.S = p;
    p += dim;
    sh.Tf = p;
    p += sg.chain_total;
    sh.xc = p;
    p += (D + 1) * W;
    sh.inv = p;
    p += D + 1;
    if (bwd) {
        sh.G = p;
        p += dim;
        sh.Tb = p;
        p += sg.chain_total;
        sh.xbar = p;
    } else {
        sh.G = sh.Tb = sh.xbar = nullptr;
    }
    for (int m = threadIdx.x; m <= D; m += blockDim.x) sh.inv[m] = m == 0 ? T(0) : T(1) / static_cast<T>(m);

    for (int64_t b = blockIdx.x; b < paths.batch; b += gridDim.x) {
        const int64_t off = paths.offsets ? paths.offsets[b] : b * paths.length;
        const int64_t len = paths.offsets ? paths.offsets[b + 1] - off : paths.length;
        const T* xin = incr + off * W;

        // Initial state: the unit tensor, or the caller's final signature.
        if (mode & kLoadFinal) {
            const T* src = sig + b * sig_stride;
            for (uint32_t i = threadIdx.x; i < dim; i += blockDim.x) sh.S[i] = src[i];
        } else {
            for (uint32_t i = threadIdx.x; i < dim; i += blockDim.x) sh.S[i] = i == 0 ? T(1) : T(0);
        }
        __syncthreads();

        if (mode & kForward) {
            T xv = len > 0 ? load_increment(sg, xin, 0) : T(0);
            for (int64_t k = 0; k < len; ++k) {
                set_increment(sg, sh, xv);
                if (k + 1 < len) xv = load_increment(sg, xin, k + 1);
                __syncthreads();
                forward_step(sg, sh);
            }
            if (sig && !(mode & kLoadFinal)) {
                T* dst = sig + b * sig_stride;
                for (uint32_t i = threadIdx.x; i < dim; i += blockDim.x) dst[i] = sh.S[i];
            }
        }
        if (bwd) {
            const T* sd = seed + b * seed_stride;
            for (uint32_t i = threadIdx.x; i < dim; i += blockDim.x) sh.G[i] = sd[i];
            T* gout = grad + off * W;
            T xv = len > 0 ? load_increment(sg, xin, len - 1) : T(0);
            __syncthreads();
            for (int64_t k = len - 1; k >= 0; --k) {
                set_increment(sg, sh, xv);
                if (k > 0) xv = load_increment(sg, xin, k - 1);
                __syncthreads();
                backward_step(sg, sh, gout + k * W);
            }
        }
        __syncthreads();
    }
}

SigGeometry make_sig_geometry(const Geometry& g) {
    SigGeometry sg{};
    sg.g = g;
    uint32_t acc = 0;
    for (int j = 0; j <= g.depth; ++j) {
        sg.choff[j] = acc;
        if (j < g.depth) acc += static_cast<uint32_t>(g.depth - j) * g.pw[j];
    }
    sg.chain_total = acc;
    return sg;
}

template <typename T>
size_t sig_smem_bytes(const SigGeometry& sg, int threads, bool bwd) {
    const size_t D = sg.g.depth, W = sg.g.width;
    size_t n = sg.g.dim + sg.chain_total + (D + 1) * W + (D + 1);
    if (bwd) n += sg.g.dim + sg.chain_total + static_cast<size_t>(threads) * W;
    return n * sizeof(T);
}

}  // namespace

template <typename T>
cudaError_t launch_signature(const Geometry& g, const DeviceInfo& dev, cudaStream_t s,
                             const T* incr, PathBatch paths, T* sig, int64_t sig_stride,
                             const T* seed, int64_t seed_stride, T* grad, bool forward) {
    if (paths.batch <= 0) return cudaSuccess;
    const SigGeometry sg = make_sig_geometry(g);
    int mode = 0;
    if (forward) {
        mode |= kForward;
        if (seed && grad) mode |= kBackward;
    } else {
        mode |= kBackward | kLoadFinal;
    }
    const bool bwd = mode & kBackward;
    constexpr auto kernel = k_signature<T>;
    cudaError_t err = allow_large_smem<kernel>(dev);
    if (err != cudaSuccess) return err;
    const int threads = threads_for(g.pw[g.depth]);
    // every (degree, letter) pair of the scaled increment needs its own thread
    if (threads < g.depth * g.width) return cudaErrorInvalidConfiguration;
    const size_t smem = sig_smem_bytes<T>(sg, threads, bwd);
    if (smem > static_cast<size_t>(dev.max_smem_optin)) return cudaErrorInvalidConfiguration;
    dim3 grid;
    if ((err = batch_grid(kernel, dev, threads, smem, paths.batch, grid)) != cudaSuccess) return err;
    kernel<<<grid, threads, smem, s>>>(sg, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
    return cudaGetLastError();
}

template cudaError_t launch_signature<float>(const Geometry&, const DeviceInfo&, cudaStream_t, const float*,
                                             PathBatch, float*, int64_t, const float*, int64_t, float*,
                                             bool);
template cudaError_t launch_signature<double>(const Geometry&, const DeviceInfo&, cudaStream_t,
                                              const double*, PathBatch, double*, int64_t, const double*,
                                              int64_t, double*, bool);

}  // namespace rpp_gb
