// signature.cu -- fused signature forward / reverse kernels.
//
// One CTA owns one path at a time (grid-stride over the batch) and keeps the
// running signature in shared memory for all of the path's increments; the
// reference's caller instead launches ft_fmexp once per increment and
// round-trips the whole state through global memory every step
// (tests/rpp/gpu/block/ops/ft_fmexp_tests.cu:126-147).
//
// Chen step S <- S (x) exp(x) for a degree-one increment x (the case of
// include/rpp/operations/intermediate/ft_fmexp.hpp:66-87 with the exponent in
// degree one).  For each level n the Horner chain
//     T^n_0 = S_0,   T^n_j = S_j + T^n_{j-1} (x) x c_{n,j},   c_{n,j} = 1/(n-j+1)
// ends in S_n <- T^n_n and costs sum_j W^j FMAs, so one step costs
// F = sum_{i=1..D} (D-i+1) W^i FMAs.  Stage j computes every chain's T^n_j at
// once from the old levels (one barrier per stage); the last stage updates all
// levels together.
//
// Reverse pass for loss = <seed, S_L>.  With G = dloss/dS_k:
//  * Phase A recovers the prefix S_{k-1} bottom-up, S_j = S'_j - T^j_{j-1} (x) x,
//    rebuilding the forward chains on the way.  The top level S_D is never read
//    by any chain (they stop at level D-1), so it is not recovered.
//  * Phase B transposes the chains top-down with scaled cotangents
//    Gh^n_j = c_{n,j} dloss/dT^n_j (Gh^n_n = G_n):
//        Gh^n_{j-1}[u] = sum_a Gh^n_j[ua] x_a c_{n,j-1}
//        xbar_a       += sum_u Gh^n_j[ua] T^n_{j-1}[u]
//    and G_{k-1,i} = G_i + sum_{n>i} (n-i+1) Gh^n_i.  G's top level never
//    changes (no chain feeds it), so it stays the seed's top level.
// Work per increment: F (forward) + F - W^D (phase A) + ~2F (phase B), nothing
// stored per step.
//
// Shared memory (elements of T): S levels 0..D-1 | top level (S_D in the
// forward, the seed's top level in the reverse pass) | G levels 0..D-1 |
// forward chains | cotangent chains | scaled increments | 1/m | one partial
// sum per thread.
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

enum SigMode : int { kForward = 1, kBackward = 2, kLoadFinal = 4, kTopLevel = 8 };

template <typename T>
struct SigShared {
    T* S;     // levels 0..D-1, followed by the top region
    T* top;   // S_D (forward) / seed top level (reverse)
    T* G;     // cotangent levels 0..D-1
    T* Tf;    // forward chains
    T* Tb;    // scaled cotangent chains
    T* xc;    // xc[m*W + a] = x_a / m, m = 1..D
    T* inv;   // inv[m] = 1/m
    T* part;  // one partial sum per thread
};

// Width either fixed at compile time (WT > 0) or read from the geometry.
template <int WT>
struct Width {
    uint32_t w;
    FastDiv fd;
    __device__ explicit Width(const Geometry& g) : w(WT > 0 ? WT : g.width), fd(g.divw) {}
    __device__ __forceinline__ uint32_t value() const { return WT > 0 ? WT : w; }
    __device__ __forceinline__ void divmod(uint32_t u, uint32_t& q, uint32_t& a) const {
        if constexpr (WT > 0) {
            q = u / WT;
            a = u % WT;
        } else {
            fd.divmod(u, q, a);
        }
    }
};

template <typename T>
__device__ __forceinline__ T* chain(const SigGeometry& sg, T* base, int n, int j) {
    return base + sg.choff[j] + static_cast<uint32_t>(n - j - 1) * sg.g.pw[j];
}

// Threads t < D*W each hold one scaled increment coefficient.
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
    if (t < static_cast<uint32_t>(sg.g.depth) * W) return __ldg(path_incr + k * W + t % W);
    return T(0);
}

// S <- S (x) exp(x).  `top` = false leaves level D (and its chains) alone.
// Ends with a barrier.
template <typename T, int WT>
__device__ void forward_step(const SigGeometry& sg, const SigShared<T>& sh, bool top) {
    const Geometry& G = sg.g;
    const Width<WT> Wd(G);
    const uint32_t W = Wd.value();
    const int D = G.depth;
    const int nmax = top ? D : D - 1;
    T* S = sh.S;
    const T s0 = S[0];
    for (int j = 1; j < nmax; ++j) {
        const uint32_t wj = G.pw[j];
        const T* Sj = S + G.db[j];
        for (int n = j + 1; n <= nmax; ++n) {
            T* dst = chain(sg, sh.Tf, n, j);
            const T* prev = chain(sg, sh.Tf, n, j - 1);
            const T* xm = sh.xc + (n - j + 1) * W;
#pragma unroll 4
            for (uint32_t u = threadIdx.x; u < wj; u += blockDim.x) {
                uint32_t q, a;
                Wd.divmod(u, q, a);
                const T p = j == 1 ? s0 : prev[q];
                dst[u] = fma(p, xm[a], Sj[u]);
            }
        }
        __syncthreads();
    }
    const T* x1 = sh.xc + W;
    for (int n = 1; n <= nmax; ++n) {
        const uint32_t wn = G.pw[n];
        T* Sn = S + G.db[n];
        const T* prev = chain(sg, sh.Tf, n, n - 1);
#pragma unroll 4
        for (uint32_t u = threadIdx.x; u < wn; u += blockDim.x) {
            uint32_t q, a;
            Wd.divmod(u, q, a);
            const T p = n == 1 ? s0 : prev[q];
            Sn[u] = fma(p, x1[a], Sn[u]);
        }
    }
    __syncthreads();
}

// One reverse step: S_k -> S_{k-1} below the top level, G_k -> G_{k-1},
// grad_k <- xbar.  Ends with a barrier.
template <typename T, int WT>
__device__ void backward_step(const SigGeometry& sg, const SigShared<T>& sh, T* grad_k) {
    const Geometry& G = sg.g;
    const Width<WT> Wd(G);
    const uint32_t W = Wd.value();
    const int D = G.depth;
    T* S = sh.S;
    const T s0 = S[0];
    const T* x1 = sh.xc + W;

    // Phase A: recover S_1..S_{D-1} of the prefix and the forward chains.
    for (int j = 1; j < D; ++j) {
        const uint32_t wj = G.pw[j];
        T* Sj = S + G.db[j];
        const T* own = chain(sg, sh.Tf, j, j - 1);
#pragma unroll 2
        for (uint32_t u = threadIdx.x; u < wj; u += blockDim.x) {
            uint32_t q, a;
            Wd.divmod(u, q, a);
            const T s = fma(-(j == 1 ? s0 : own[q]), x1[a], Sj[u]);
            Sj[u] = s;
            for (int n = j + 1; n <= D; ++n) {
                const T p = j == 1 ? s0 : chain(sg, sh.Tf, n, j - 1)[q];
                chain(sg, sh.Tf, n, j)[u] = fma(p, sh.xc[(n - j + 1) * W + a], s);
            }
        }
        __syncthreads();
    }

    // Phase B: scaled cotangent chains, top stage first.  xbar partials are
    // letter-specialised: thread t accumulates letter t % W only, so each
    // thread keeps a single partial sum.
    const uint32_t slots = blockDim.x / W;
    const uint32_t my_a = threadIdx.x % W, my_slot = threadIdx.x / W;
    const bool xbar_lane = my_slot < slots;
    T xacc = T(0);
    for (int j = D; j >= 2; --j) {
        const uint32_t wjm1 = G.pw[j - 1];
        // cotangent contraction Gh^n_{j-1}[u] = sum_a Gh^n_j[ua] x_a / (n-j+2)
        for (int n = j; n <= D; ++n) {
            const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
            T* gout = chain(sg, sh.Tb, n, j - 1);
            const T* xm = sh.xc + (n - j + 2) * W;
#pragma unroll 2
            for (uint32_t u = threadIdx.x; u < wjm1; u += blockDim.x) {
                const T* row = gin + u * W;
                T acc = T(0);
                if constexpr (WT > 0) {
#pragma unroll
                    for (int a = 0; a < WT; ++a) acc = fma(row[a], xm[a], acc);
                } else {
                    for (uint32_t a = 0; a < W; ++a) acc = fma(row[a], xm[a], acc);
                }
                gout[u] = acc;
            }
        }
        // xbar_a += sum_u Gh^n_j[ua] T^n_{j-1}[u]
        if (xbar_lane) {
            for (int n = j; n <= D; ++n) {
                const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                const T* tprev = chain(sg, sh.Tf, n, j - 1);
#pragma unroll 4
                for (uint32_t u = my_slot; u < wjm1; u += slots) xacc = fma(gin[u * W + my_a], tprev[u], xacc);
            }
        }
        __syncthreads();
    }

    // Stage 1 (xbar_a += Gh^n_1[a] S_0) is folded into the reduction.  Thread
    // a < W reads G_1[a] here before it updates that same element below.
    T v1 = T(0);
    if (threadIdx.x < W) {
        const uint32_t a = threadIdx.x;
        for (int n = 1; n <= D; ++n) {
            const T* g1 = n == 1 ? (D == 1 ? sh.top : sh.G + G.db[1]) : chain(sg, sh.Tb, n, 1);
            v1 = fma(g1[a], s0, v1);
        }
    }
    sh.part[threadIdx.x] = xbar_lane ? xacc : T(0);
    // G_{k-1,i} = G_i + sum_{n>i} (n-i+1) Gh^n_i for 1 <= i < D (G_0 is never
    // used).  Level-1 element u is updated by thread u (W <= blockDim.x).
    for (int i = 1; i < D; ++i) {
        const uint32_t wi = G.pw[i];
        T* Gi = sh.G + G.db[i];
        for (uint32_t u = threadIdx.x; u < wi; u += blockDim.x) {
            T s = Gi[u];
            for (int n = i + 1; n <= D; ++n) s = fma(static_cast<T>(n - i + 1), chain(sg, sh.Tb, n, i)[u], s);
            Gi[u] = s;
        }
    }
    __syncthreads();
    if (threadIdx.x < W) {
        const uint32_t a = threadIdx.x;
        T v = v1;
        for (uint32_t s = 0; s < slots; ++s) v += sh.part[s * W + a];
        grad_k[a] = v;
    }
    __syncthreads();
}

template <typename T, int WT>
__global__ void __launch_bounds__(256) k_signature(SigGeometry sg, const T* __restrict__ incr, PathBatch paths,
                                                   T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                                                   T* grad, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t dim = G.dim;
    const uint32_t lo = G.db[D];  // coefficients below the top level
    const bool bwd = mode & kBackward;
    const bool fwd_top = mode & kTopLevel;

    SigShared<T> sh;
    T* p = reinterpret_cast<T*>(smem_raw);
    sh.S = p;
    sh.top = p + lo;
    p += dim;
    sh.Tf = p;
    p += sg.chain_total;
    sh.xc = p;
    p += (D + 1) * W;
    sh.inv = p;
    p += D + 1;
    sh.part = p;
    p += blockDim.x;
    if (bwd) {
        sh.G = p;
        p += lo;
        sh.Tb = p;
    } else {
        sh.G = sh.Tb = nullptr;
    }
    for (int m = threadIdx.x; m <= D; m += blockDim.x) sh.inv[m] = m == 0 ? T(0) : T(1) / static_cast<T>(m);

    for (int64_t b = blockIdx.x; b < paths.batch; b += gridDim.x) {
        const int64_t off = paths.offsets ? paths.offsets[b] : b * paths.length;
        const int64_t len = paths.offsets ? paths.offsets[b + 1] - off : paths.length;
        const T* xin = incr + off * W;

        if (mode & kLoadFinal) {
            const T* src = sig + b * sig_stride;
            for (uint32_t i = threadIdx.x; i < lo; i += blockDim.x) sh.S[i] = src[i];
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
                forward_step<T, WT>(sg, sh, fwd_top);
            }
            if (sig && !(mode & kLoadFinal)) {
                T* dst = sig + b * sig_stride;
                for (uint32_t i = threadIdx.x; i < dim; i += blockDim.x) dst[i] = sh.S[i];
            }
            __syncthreads();
        }
        if (bwd) {
            const T* sd = seed + b * seed_stride;
            for (uint32_t i = threadIdx.x; i < lo; i += blockDim.x) sh.G[i] = sd[i];
            for (uint32_t i = threadIdx.x; i < G.pw[D]; i += blockDim.x) sh.top[i] = sd[lo + i];
            T* gout = grad + off * W;
            T xv = len > 0 ? load_increment(sg, xin, len - 1) : T(0);
            __syncthreads();
            for (int64_t k = len - 1; k >= 0; --k) {
                set_increment(sg, sh, xv);
                if (k > 0) xv = load_increment(sg, xin, k - 1);
                __syncthreads();
                backward_step<T, WT>(sg, sh, gout + k * W);
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
    size_t n = sg.g.dim + sg.chain_total + (D + 1) * W + (D + 1) + threads;
    if (bwd) n += sg.g.db[D] + sg.chain_total;
    return n * sizeof(T);
}

template <typename T, int WT>
cudaError_t launch_width(const SigGeometry& sg, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                         PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride, T* grad,
                         int mode) {
    constexpr auto kernel = k_signature<T, WT>;
    cudaError_t err = allow_large_smem<kernel>(dev);
    if (err != cudaSuccess) return err;
    const int threads = threads_for(sg.g.pw[sg.g.depth]);
    // every (degree, letter) pair of the scaled increment needs its own thread
    if (threads < sg.g.depth * sg.g.width || threads < sg.g.width) return cudaErrorInvalidConfiguration;
    const size_t smem = sig_smem_bytes<T>(sg, threads, mode & kBackward);
    if (smem > static_cast<size_t>(dev.max_smem_optin)) return cudaErrorInvalidConfiguration;
    dim3 grid;
    if ((err = batch_grid(kernel, dev, threads, smem, paths.batch, grid)) != cudaSuccess) return err;
    kernel<<<grid, threads, smem, s>>>(sg, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
    return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_signature(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                             PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                             T* grad, bool forward) {
    if (paths.batch <= 0) return cudaSuccess;
    const SigGeometry sg = make_sig_geometry(g);
    int mode = 0;
    if (forward) {
        mode |= kForward;
        if (seed && grad) mode |= kBackward;
        // The top level of S is only an output: a gradient-only call skips it.
        if (sig) mode |= kTopLevel;
    } else {
        mode |= kBackward | kLoadFinal;
    }
    switch (g.width) {
        case 2: return launch_width<T, 2>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        case 3: return launch_width<T, 3>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        case 4: return launch_width<T, 4>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        case 5: return launch_width<T, 5>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        case 6: return launch_width<T, 6>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        case 8: return launch_width<T, 8>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        case 16: return launch_width<T, 16>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
        default: return launch_width<T, 0>(sg, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode);
    }
}

template cudaError_t launch_signature<float>(const Geometry&, const DeviceInfo&, cudaStream_t, const float*,
                                             PathBatch, float*, int64_t, const float*, int64_t, float*, bool);
template cudaError_t launch_signature<double>(const Geometry&, const DeviceInfo&, cudaStream_t, const double*,
                                              PathBatch, double*, int64_t, const double*, int64_t, double*, bool);

}  // namespace rpp_gb
