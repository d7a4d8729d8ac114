// signature_split.cu -- the fused signature kernel for states split over a
// thread-block cluster (schedule bits 28-30 = P - 1: P CTAs per path).
//
// A path's state (levels, forward chains, cotangent levels and chains) is
// divided by first letter: CTA `rank` of the cluster holds, of every level
// j >= 1, the W^j / P coefficients whose first letter lies in
// [rank W/P, (rank+1) W/P) -- so a W6 D6 FP64 state (437 KB a tensor) fits in
// the shared memory of 2, 3 or 6 CTAs instead of running from an L2-resident
// global workspace.  The per-path code is the single-CTA code on the sliced
// geometry (signature_body.cuh: forward_step / backward_step with SPLIT set,
// which offsets level-1 letters by the CTA's first letter); the only traffic
// between the CTAs is each reverse step's letter-gradient partials (W values
// per CTA, stored into rank 0's shared memory through distributed shared
// memory, split_exchange) and the task index that rank 0 broadcasts.  The
// reference keeps one whole tensor per CTA and round-trips it through global
// memory every step (include/rpp/gpu/block/operations/intermediate/
// ft_fmexp.hpp:61-83).
#include "signature_body.cuh"

namespace rpp_gb {
namespace {

// The level starts db[0..D+1] of the full (unsplit) tensor: where each
// CTA's slices go in the signature, seed and gradient rows.
struct LevelStarts {
    uint32_t db[kMaxDepth + 2];
};

// Copies levels [0, jend) between this CTA's sliced array `local` (layout of
// the sliced geometry) and a full tensor row `row` (global memory).  Level 0
// is the scalar every CTA holds; only rank 0 writes it out.
template <typename T, bool TO_ROW>
__device__ __forceinline__ void copy_levels(const CtaTeam& tm, const SigGeometry& sg, const LevelStarts& full,
                                            uint32_t rank, T* local, T* row, int jend) {
    for (int j = 0; j < jend; ++j) {
        const uint32_t n = sg.g.pw[j];
        const uint32_t lo = sg.g.db[j];
        const uint32_t go = j == 0 ? 0u : full.db[j] + rank * n;
        if (TO_ROW && j == 0 && rank != 0) continue;
        for (uint32_t u = tm.rank(); u < n; u += tm.size()) {
            if constexpr (TO_ROW)
                row[go + u] = local[lo + u];
            else
                local[lo + u] = row[go + u];
        }
    }
}

// One path b of a split cluster: forward pass, and with kBackward the
// reverse pass, as run_path; ends with a barrier of the CTA.
template <typename T, int WT>
__device__ __forceinline__ void run_path_split(const CtaTeam& tm, const SigGeometry& sg, const LevelStarts& full,
                                               SigShared<T>& sh, SplitCtx<T>& cx, const T* __restrict__ incr,
                                               int64_t b, int64_t off, int64_t len, T* sig, int64_t sig_stride,
                                               const T* seed, int64_t seed_stride, T* grad, int mode) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t lo = G.db[D];
    const bool bwd = mode & kBackward;
    const bool fwd_top = mode & kTopLevel;
    const bool top_global = mode & kTopGlobal;
    const uint32_t held = top_global ? lo : G.dim;
    const int nmax = fwd_top ? D : D - 1;
    const uint32_t top_off = full.db[D] + cx.rank * G.pw[D];  // this CTA's top-level slice in a row
    const T* xin = incr + off * W;

    for (uint32_t i = tm.rank(); i < held; i += tm.size()) sh.S[i] = i == 0 ? T(1) : T(0);
    if (top_global && fwd_top) {
        sh.top = sig + b * sig_stride + top_off;
        for (uint32_t i = tm.rank(); i < G.pw[D]; i += tm.size()) sh.top[i] = T(0);
    }
    if (len > 0) set_increment(tm, sg, sh, xc_buf(sh, 0), load_increment(tm, sg, xin, 0));
    tm.sync();
    T xv = len > 1 ? load_increment(tm, sg, xin, 1) : T(0);
    for (int64_t k = 0; k < len; ++k) {
        const T x_next = xv;
        if (k + 2 < len) xv = load_increment(tm, sg, xin, k + 2);
        forward_step<T, WT, true>(tm, sg, sh, xc_buf(sh, k), xc_buf(sh, k + 1), x_next, nmax, top_global, false);
    }
    if (sig) copy_levels<T, true>(tm, sg, full, cx.rank, sh.S, sig + b * sig_stride, top_global ? D : D + 1);
    tm.sync();
    if (bwd) {
        const T* sd = seed + b * seed_stride;
        copy_levels<T, false>(tm, sg, full, cx.rank, sh.G, const_cast<T*>(sd), D);
        if (top_global)
            sh.top = const_cast<T*>(sd) + top_off;  // read only in the reverse pass
        else
            for (uint32_t i = tm.rank(); i < G.pw[D]; i += tm.size()) sh.top[i] = sd[top_off + i];
        T* gout = grad + off * W;
        cx.gout = gout;
        cx.len = len;
        if (len > 0) set_increment(tm, sg, sh, xc_buf(sh, len - 1), load_increment(tm, sg, xin, len - 1));
        tm.sync();
        T xb = len > 1 ? load_increment(tm, sg, xin, len - 2) : T(0);
        for (int64_t k = len - 1; k >= 0; --k) {
            const T x_next = xb;
            if (k >= 2) xb = load_increment(tm, sg, xin, k - 2);
            backward_step<T, WT, true>(tm, sg, sh, xc_buf(sh, k), xc_buf(sh, k - 1), x_next,
                                       k + 1 < len ? gout : nullptr, &cx, k);
        }
        if (len > 0) split_finish(tm, sg, sh, cx);
    }
    tm.sync();
}

// Persistent clusters: rank 0 of each takes the next path (work counter for
// ragged batches, else cluster index + iteration x clusters) and broadcasts
// it to the cluster's CTAs through distributed shared memory, in a slot of
// the iteration's parity (a CTA reads slot i mod 2 before arriving on the
// barrier that precedes the next write of that slot).
// COT: the cotangent level and chains in this CTA's slice of the global
// workspace `gws` (kCotGlobal, L2-resident), the state and forward chains in
// shared memory.
template <typename T, int WT, bool COT>
__global__ void __launch_bounds__(kResidentMaxThreads, 2) k_signature_split(SigGeometry sg, LevelStarts full,
                                                                           const T* __restrict__ incr, PathBatch paths,
                                                                           T* sig, int64_t sig_stride, const T* seed,
                                                                           int64_t seed_stride, T* grad, int mode,
                                                                           T* gws, int64_t gws_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int64_t s_next[2];
    const CtaTeam tm;
    bool vec4 = false;
    SigShared<T> sh = place_arrays<T, WT, COT>(tm, sg, mode, gws, gws_stride, smem_raw, vec4);
    uint32_t P;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(P));
    const uint32_t rank = cluster_rank();
    sh.lofs = rank * (static_cast<uint32_t>(sg.g.width) / P);
    SplitCtx<T> cx{sh.part + tm.size(), P, rank, nullptr, 0};
    const int64_t cluster = blockIdx.x / P, clusters = gridDim.x / P;
    // every CTA of the cluster has started before any distributed access
    cluster_arrive();
    cluster_wait();
    for (int64_t it = 0;; ++it) {
        if (rank == 0 && threadIdx.x == 0) {
            const int64_t next = paths.counter ? static_cast<int64_t>(atomicAdd(paths.counter, 1u))
                                               : cluster + it * clusters;
            for (uint32_t r = 0; r < P; ++r) store_remote(&s_next[it & 1], r, next);
        }
        cluster_arrive();
        cluster_wait();
        const int64_t slot = s_next[it & 1];
        if (slot >= paths.batch) break;
        const int64_t b = paths.order ? paths.order[slot] : slot;
        const int64_t off = paths.offsets ? paths.offsets[b] : b * paths.length;
        const int64_t len = paths.offsets ? paths.offsets[b + 1] - off : paths.length;
        run_path_split<T, WT>(tm, sg, full, sh, cx, incr, b, off, len, sig, sig_stride, seed, seed_stride, grad,
                              mode);
    }
}

// The sliced geometry of one CTA of P: level j >= 1 keeps W^j / P
// coefficients; the width (and its divider) is the full tensor's.
SigGeometry sliced_geometry(const Geometry& g, int P) {
    Geometry s = g;
    uint32_t db = 0;
    for (int j = 0; j <= g.depth; ++j) {
        s.pw[j] = j == 0 ? 1u : g.pw[j] / static_cast<uint32_t>(P);
        s.db[j] = db;
        db += s.pw[j];
    }
    s.db[g.depth + 1] = db;
    s.pw[g.depth + 1] = 0;
    s.dim = db;
    return make_sig_geometry(s);
}

template <typename T, int WT, bool COT>
cudaError_t launch_split_kernel(const SigGeometry& sg, const LevelStarts& full, const DeviceInfo& dev,
                                cudaStream_t s, const T* incr, PathBatch paths, T* sig, int64_t sig_stride,
                                const T* seed, int64_t seed_stride, T* grad, int mode, int threads, int P);

template <typename T, int WT>
cudaError_t launch_split_width(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                               PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                               T* grad, int mode, int threads, int P) {
    const SigGeometry sg = sliced_geometry(g, P);
    LevelStarts full{};
    for (int j = 0; j <= g.depth + 1; ++j) full.db[j] = g.db[j];
    const bool cot = (mode & kCotGlobal) && (mode & kBackward);
    if (cot) return launch_split_kernel<T, WT, true>(sg, full, dev, s, incr, paths, sig, sig_stride, seed, seed_stride,
                                                     grad, mode, threads, P);
    return launch_split_kernel<T, WT, false>(sg, full, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad,
                                             mode & ~kCotGlobal, threads, P);
}

template <typename T, int WT, bool COT>
cudaError_t launch_split_kernel(const SigGeometry& sg, const LevelStarts& full, const DeviceInfo& dev,
                                cudaStream_t s, const T* incr, PathBatch paths, T* sig, int64_t sig_stride,
                                const T* seed, int64_t seed_stride, T* grad, int mode, int threads, int P) {
    const Geometry& g = sg.g;
    constexpr auto kernel = k_signature_split<T, WT, COT>;
    cudaError_t err = allow_large_smem<kernel>(dev);
    if (err != cudaSuccess) return err;
    cudaFuncAttributes attr{};
    if ((err = cudaFuncGetAttributes(&attr, kernel)) != cudaSuccess) return err;
    const size_t optin = static_cast<size_t>(dev.max_smem_optin) - attr.sharedSizeBytes;
    // with COT the cotangent arrays are not in shared memory
    const bool bwd_smem = (mode & kBackward) && !COT;
    const size_t slots = 2 * static_cast<size_t>(P) * g.width * sizeof(T);
    size_t smem = sig_smem_bytes<T>(sg, threads, bwd_smem, true, mode & kTopGlobal) + slots;
    if (smem > optin && !(mode & kTopGlobal)) {
        mode |= kTopGlobal;
        smem = sig_smem_bytes<T>(sg, threads, bwd_smem, true, true) + slots;
    }
    if (smem > optin) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attrs[1];
    attrs[0].id = cudaLaunchAttributeClusterDimension;
    attrs[0].val.clusterDim.x = static_cast<unsigned>(P);
    attrs[0].val.clusterDim.y = 1;
    attrs[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(static_cast<unsigned>(threads));
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attrs;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(static_cast<unsigned>(P) * static_cast<unsigned>(std::max(1, dev.sm_count)));
    int clusters = 0;
    if ((err = cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg)) != cudaSuccess) return err;
    if (clusters < 1) return cudaErrorInvalidConfiguration;
    const int64_t n = std::max<int64_t>(1, std::min<int64_t>(paths.batch, clusters));
    cfg.gridDim = dim3(static_cast<unsigned>(n * P));
    if constexpr (!COT) {
        return cudaLaunchKernelEx(&cfg, kernel, sg, full, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode,
                                  static_cast<T*>(nullptr), int64_t{0});
    } else {
        // the cotangent level (below the top) and chains of each CTA, in a
        // stream-ordered workspace released after the launch
        const int64_t stride = static_cast<int64_t>((sg.g.db[sg.g.depth] + sg.chain_total + 31) / 32 * 32);
        T* ws = nullptr;
        err = cudaMallocAsync(reinterpret_cast<void**>(&ws), static_cast<size_t>(n * P) * stride * sizeof(T), s);
        if (err != cudaSuccess) return err;
        err = cudaLaunchKernelEx(&cfg, kernel, sg, full, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode,
                                 ws, stride);
        cudaError_t ferr = cudaFreeAsync(ws, s);
        return err != cudaSuccess ? err : ferr;
    }
}

}  // namespace

template <typename T>
cudaError_t launch_signature_split(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* incr,
                                   PathBatch paths, T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                                   T* grad, int mode, int threads, int P) {
    if (P < 2 || P > 8 || g.width % P != 0 || g.depth < 2) return cudaErrorInvalidConfiguration;
    if (mode & (kLoadFinal | kMergedReverse)) return cudaErrorInvalidConfiguration;
    if (threads % 32 != 0 || threads > kResidentMaxThreads || threads < g.depth * g.width)
        return cudaErrorInvalidConfiguration;
    switch (g.width) {
        case 2: return launch_split_width<T, 2>(g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads, P);
        case 3: return launch_split_width<T, 3>(g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads, P);
        case 4: return launch_split_width<T, 4>(g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads, P);
        case 6: return launch_split_width<T, 6>(g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads, P);
        case 8: return launch_split_width<T, 8>(g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads, P);
        default: return launch_split_width<T, 0>(g, dev, s, incr, paths, sig, sig_stride, seed, seed_stride, grad, mode, threads, P);
    }
}

template cudaError_t launch_signature_split<float>(const Geometry&, const DeviceInfo&, cudaStream_t, const float*,
                                                   PathBatch, float*, int64_t, const float*, int64_t, float*, int,
                                                   int, int);
template cudaError_t launch_signature_split<double>(const Geometry&, const DeviceInfo&, cudaStream_t, const double*,
                                                    PathBatch, double*, int64_t, const double*, int64_t, double*,
                                                    int, int, int);

}  // namespace rpp_gb
