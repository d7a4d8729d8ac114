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
// Barriers: D per forward step and 2D-1 per reverse step.  The scaled
// increments are double-buffered by step parity so refreshing them needs no
// barrier of its own, and each reverse step's G update and gradient reduction
// run inside the next step's first recovery stage.  The threads per CTA are a
// schedule parameter (chosen by the autotuner, rpp_gb_signature_tune).
//
// Shared memory (elements of T): S levels 0..D-1 | top level (S_D in the
// forward, the seed's top level in the reverse pass) | forward chains | 2 x
// scaled increments | 1/m | one partial per thread | G levels 0..D-1 |
// cotangent chains.
#include <mutex>
#include <type_traits>

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

// kTopGlobal: the top level lives in global memory -- S_D in the output
// signature row during the forward pass, the seed's top level read from the
// seed row in the reverse pass -- so a state that misses shared memory by
// less than one level (W2 D12 FP64: 229 KB, 196 KB without its top) still
// runs resident.  Level D is only ever updated by the thread that owns the
// coefficient, so no barrier orders these accesses.
// kMergedReverse: reverse steps by backward_step_merged (D barriers) instead
// of backward_step (2D - 1).
enum SigMode : int {
    kForward = 1,
    kBackward = 2,
    kLoadFinal = 4,
    kTopLevel = 8,
    kTopGlobal = 16,
    kCotGlobal = 32,
    kMergedReverse = 64
};

template <typename T>
struct SigShared {
    T* S;     // levels 0..D-1, followed by the top region
    T* top;   // S_D (forward) / seed top level (reverse)
    T* G;     // cotangent levels 0..D-1
    T* Tf;    // forward chains
    T* Tb;    // scaled cotangent chains
    T* xc;    // two buffers of (D+1)*W: xc[m*W + a] = x_a / m, m = 1..D
    T* inv;   // inv[m] = 1/m
    T* num;   // num[m] = m (the G update's integer weights, read instead of converted)
    T* part;  // one partial sum per thread
    uint32_t xcs;  // size of one increment buffer
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

template <typename T>
__device__ __forceinline__ T* xc_buf(const SigShared<T>& sh, int64_t k) {
    return sh.xc + (k & 1) * sh.xcs;
}

// Threads t < D*W each hold one scaled increment coefficient.
template <typename T>
__device__ __forceinline__ void set_increment(const SigGeometry& sg, const SigShared<T>& sh, T* xc, T xv) {
    const uint32_t W = static_cast<uint32_t>(sg.g.width);
    const uint32_t t = threadIdx.x;
    if (t < static_cast<uint32_t>(sg.g.depth) * W) {
        const uint32_t m = 1 + t / W;
        xc[m * W + t % W] = xv * sh.inv[m];
    }
}

template <typename T>
__device__ __forceinline__ T load_increment(const SigGeometry& sg, const T* path_incr, int64_t k) {
    const uint32_t W = static_cast<uint32_t>(sg.g.width);
    const uint32_t t = threadIdx.x;
    if (t < static_cast<uint32_t>(sg.g.depth) * W) return __ldg(path_incr + k * W + t % W);
    return T(0);
}

// Row mode (reverse pass).  A level-j array splits into W^{j-1} rows of W
// consecutive coefficients (prefix word, then the last letter), and every
// chain link multiplies a row by one prefix coefficient.  With W fixed at
// compile time one thread takes a whole row: W FMAs per prefix coefficient
// loaded, with no index split per coefficient.
//  * Phase B (kRowModeB): the cotangent chains of one stage form one run of
//    rows, offsets carried from chain to chain so warps stay full, with the
//    scaled increment in registers.
//  * Phase A (kRowModeA): the recovery of S_j and of the chain links T^n_j
//    row by row, in stages with at least kRowMin rows (a warp instruction
//    occupies the FP64 pipe for the same time however few of its lanes are
//    active, so smaller stages keep one thread per coefficient).  Rows are
//    W elements apart, so W = 4 and 8 (4- and 8-way shared-memory bank
//    conflicts on 8-byte rows) keep one thread per coefficient too.
// The forward step keeps one thread per coefficient: measured on W5 D5 and
// W2 D12, row mode there was slower.
template <int WT>
constexpr bool kRowModeB = WT > 0 && WT <= 8;
template <int WT>
constexpr bool kRowModeA = WT == 2 || WT == 3 || WT == 5 || WT == 6 || WT == 7;
constexpr uint32_t kRowMin = 32;
// Phase B's letter gradients fused into the row loop (store_letter_partials):
// the row is read once, but every thread keeps WT accumulators and each
// reverse step ends with a butterfly of about 2 WT adds, against log2(32/W)
// for the letter-specialised loop.  Measured against that loop on fused
// forward + reverse launches: W2 D12 +12.8 %, W3 D8 +7.1 %, W6 D6 +5.8 %,
// W4 D6 equal, W5 D5 -7 % and W8 D4 -7.5 % (the butterfly's adds are 4-6 % of
// a thread's FMAs per step there).  Widths without an instantiation (WT = 0)
// keep the generic loop.
template <int WT>
constexpr bool kFusedLetters = kRowModeB<WT> && (WT == 2 || WT == 3 || WT == 6);

template <typename T, int WT>
__device__ __forceinline__ void load_row(T (&r)[WT], const T* src) {
#pragma unroll
    for (int a = 0; a < WT; ++a) r[a] = src[a];
}

// FP32 forward step four coefficients at a time (W a multiple of 4, state in
// shared memory).  In FP32 the element loop is bound by instruction issue and
// shared-memory wavefronts, not by the FMA pipe: an index split, three loads
// and a store per FMA.  Four consecutive coefficients of a level share their
// prefix coefficient and take four consecutive increment letters, so one
// thread does them with 16-byte loads and stores.  Alignment: level n >= 1
// starts at db[n] = 1 (mod 4) for W = 0 (mod 4), so the state array is placed
// with S + 1 on a 16-byte boundary; chain links of stages j >= 1 lie multiples
// of W apart from Tf + choff[1], which is placed on a 16-byte boundary too, and
// so are the scaled increments.
template <typename T, int WT>
constexpr bool kVec4 = std::is_same<T, float>::value && WT > 0 && WT % 4 == 0;

// One forward step S <- S (x) exp(x).  `nmax` = D when the top level is
// maintained, D-1 when it is not needed (gradient-only calls).  Ends with a
// barrier, after which xc_next holds the next step's scaled increment.
template <typename T, int WT>
__device__ __forceinline__ void forward_step(const SigGeometry& sg, const SigShared<T>& sh, const T* xc,
                                             T* xc_next, T x_next, int nmax, bool top_global, bool vec4) {
    const Geometry& G = sg.g;
    const Width<WT> Wd(G);
    const uint32_t W = Wd.value();
    T* S = sh.S;
    const T s0 = S[0];
    // Each stage's chains (and then the levels of the last stage) form one
    // run of coefficients: a thread that passes the end of one chain carries
    // its offset into the next, so the small chains and levels are spread
    // over the warps instead of all starting at warp 0.
    for (int j = 1; j < nmax; ++j) {
        const uint32_t wj = G.pw[j];
        const T* Sj = S + G.db[j];
        if constexpr (kVec4<T, WT>) {
            if (vec4) {
                uint32_t v = threadIdx.x;  // groups of four coefficients
                for (int n = j + 1; n <= nmax; ++n) {
                    const T* prev = chain(sg, sh.Tf, n, j - 1);
                    float4* dst = reinterpret_cast<float4*>(chain(sg, sh.Tf, n, j));
                    const T* xm = xc + (n - j + 1) * WT;
                    const uint32_t groups = wj / 4;
                    for (; v < groups; v += blockDim.x) {
                        const uint32_t u = 4 * v, q = u / WT, a = u % WT;
                        const T pq = j == 1 ? s0 : prev[q];
                        const float4 sv = reinterpret_cast<const float4*>(Sj)[v];
                        const float4 xv = *reinterpret_cast<const float4*>(xm + a);
                        dst[v] = make_float4(fmaf(pq, xv.x, sv.x), fmaf(pq, xv.y, sv.y), fmaf(pq, xv.z, sv.z),
                                             fmaf(pq, xv.w, sv.w));
                    }
                    v -= groups;
                }
                __syncthreads();
                continue;
            }
        }
        uint32_t u = threadIdx.x;
        for (int n = j + 1; n <= nmax; ++n) {
            T* dst = chain(sg, sh.Tf, n, j);
            const T* prev = chain(sg, sh.Tf, n, j - 1);
            const T* xm = xc + (n - j + 1) * W;
            for (; u < wj; u += blockDim.x) {
                uint32_t q, a;
                Wd.divmod(u, q, a);
                const T p = j == 1 ? s0 : prev[q];
                dst[u] = fma(p, xm[a], Sj[u]);
            }
            u -= wj;
        }
        __syncthreads();
    }
    const T* x1 = xc + W;
    int n_first = 1;
    if constexpr (kVec4<T, WT>) {
        if (vec4) {  // (top level in shared memory)
            uint32_t v = threadIdx.x;
            for (int n = 1; n <= nmax; ++n) {
                const T* prev = chain(sg, sh.Tf, n, n - 1);
                float4* Sn = reinterpret_cast<float4*>(S + G.db[n]);
                const uint32_t groups = G.pw[n] / 4;
                for (; v < groups; v += blockDim.x) {
                    const uint32_t u = 4 * v, q = u / WT, a = u % WT;
                    const T pq = n == 1 ? s0 : prev[q];
                    const float4 xv = *reinterpret_cast<const float4*>(x1 + a);
                    float4 sv = Sn[v];
                    sv.x = fmaf(pq, xv.x, sv.x);
                    sv.y = fmaf(pq, xv.y, sv.y);
                    sv.z = fmaf(pq, xv.z, sv.z);
                    sv.w = fmaf(pq, xv.w, sv.w);
                    Sn[v] = sv;
                }
                v -= groups;
            }
            n_first = nmax + 1;
        }
    }
    uint32_t v = threadIdx.x;
    for (int n = n_first; n <= nmax; ++n) {
        const uint32_t wn = G.pw[n];
        T* Sn = n == G.depth ? sh.top : S + G.db[n];
        const T* prev = chain(sg, sh.Tf, n, n - 1);
        if (n == G.depth && top_global) {
            // S_D in global memory: four independent read-modify-writes per
            // batch, so their L2 latencies overlap (each coefficient is owned
            // by one thread for the whole path)
            const uint32_t bd = blockDim.x;
            for (uint32_t u0 = threadIdx.x; u0 < wn; u0 += 4 * bd) {
                T v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t u = u0 + k * bd;
                    v[k] = u < wn ? Sn[u] : T(0);
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t u = u0 + k * bd;
                    if (u < wn) {
                        uint32_t q, a;
                        Wd.divmod(u, q, a);
                        Sn[u] = fma(n == 1 ? s0 : prev[q], x1[a], v[k]);
                    }
                }
            }
            continue;
        }
        for (; v < wn; v += blockDim.x) {
            uint32_t q, a;
            Wd.divmod(v, q, a);
            const T p = n == 1 ? s0 : prev[q];
            Sn[v] = fma(p, x1[a], Sn[v]);
        }
        v -= wn;
    }
    set_increment(sg, sh, xc_next, x_next);
    __syncthreads();
}

// Partial letter gradients of one reverse step.  Thread t accumulated letter
// t mod W; lanes of a warp with the same letter (lanes l, l + W, l + 2W, ...)
// are summed by a shuffle tree, and lane l < W of warp w stores the warp's
// partial of letter (32w + l) mod W at part[w*W + letter] -- log2(32/W) adds
// per warp instead of W threads each adding blockDim/W partials in sequence.
// W > 16 keeps one partial per thread (part[t]).  partial_groups() gives the
// number of partials per letter either way.
template <typename T>
__device__ __forceinline__ void store_partials(const SigShared<T>& sh, T v, uint32_t W) {
    if (W > 16) {
        sh.part[threadIdx.x] = v;
        return;
    }
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t off = W; off < 32u; off *= 2u) {
        const T o = __shfl_down_sync(0xffffffffu, v, off);
        if (lane + off < 32u) v += o;
    }
    if (lane < W) sh.part[(threadIdx.x >> 5) * W + threadIdx.x % W] = v;
}

__device__ __forceinline__ uint32_t partial_groups(uint32_t W) { return W > 16 ? blockDim.x / W : blockDim.x / 32; }

// Row mode's letter partials: every thread holds an accumulator per letter
// (xa[a]), and the warp's totals go to part[w*W + a], the layout of
// store_partials.  A reduce-scatter butterfly: at offset 16 the lower half of
// the warp keeps letters [0, h) of its pair's sums and the upper half
// [h, WT), h = ceil(WT/2), so each level halves the letters a lane holds (a
// shorter range padded with zeros: `cnt` counts the real letters from
// `base`); once one is left, plain xor levels finish the sum.  WT = 5 takes 8
// shuffles and 8 adds, where a separate reduction per letter takes 25 of each.
template <typename T, int K>
__device__ __forceinline__ void letter_butterfly(T (&v)[K], uint32_t lane, uint32_t off, uint32_t& base,
                                                 uint32_t& cnt) {
    if constexpr (K > 1) {
        constexpr int h = (K + 1) / 2;
        const bool upper = (lane & off) != 0;
        T next[h];
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const T hi = h + i < K ? v[h + i] : T(0);
            const T send = upper ? v[i] : hi;
            const T keep = upper ? hi : v[i];
            next[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
        if (upper) {
            base += h;
            cnt = cnt > static_cast<uint32_t>(h) ? cnt - h : 0u;
        } else if (cnt > static_cast<uint32_t>(h)) {
            cnt = h;
        }
        letter_butterfly<T, h>(next, lane, off >> 1, base, cnt);
        v[0] = next[0];
    } else {
        for (; off > 0; off >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], off);
    }
}

template <typename T, int WT>
__device__ __forceinline__ void store_letter_partials(const SigShared<T>& sh, T (&xa)[WT]) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0, cnt = WT;
    letter_butterfly<T, WT>(xa, lane, 16u, base, cnt);
    // lanes that differ only in the bits of the plain xor levels hold the same
    // total; the one with those bits zero stores it
    constexpr uint32_t halvings = WT <= 1 ? 0u : WT <= 2 ? 1u : WT <= 4 ? 2u : WT <= 8 ? 3u : 4u;
    if (cnt > 0u && (lane & ((32u >> halvings) - 1u)) == 0u)
        sh.part[(threadIdx.x >> 5) * WT + base] = xa[0];
}

// Finish a reverse step: grad_k from the partials (the stage-1 terms
// sum_n Gh^n_1[a] S_0 folded in) and, when `update_g`, G_{k-1} from the
// cotangent chains.  Runs between barriers, beside the first recovery stage,
// which runs on warp 0: the W gradient lanes are the first W threads of the
// CTA's last warp(s), and each of them updates G_1[a] after reading it.  The
// other levels of G form one run of coefficients over all threads.
template <typename T>
__device__ __forceinline__ void finish_reverse_step(const SigGeometry& sg, const SigShared<T>& sh, T* grad_k,
                                                    bool update_g, uint32_t groups, bool update_upper = true) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const T s0 = sh.S[0];
    const uint32_t gl = blockDim.x - ((W + 31u) & ~31u);  // (blockDim.x >= W, both multiples of 32 after rounding)
    if (threadIdx.x >= gl && threadIdx.x < gl + W) {
        const uint32_t a = threadIdx.x - gl;
        T v = T(0);
        for (int n = 1; n <= D; ++n) {
            const T* g1 = n == 1 ? (D == 1 ? sh.top : sh.G + G.db[1]) : chain(sg, sh.Tb, n, 1);
            v = fma(g1[a], s0, v);
        }
        for (uint32_t s = 0; s < groups; ++s) v += sh.part[s * W + a];
        grad_k[a] = v;
        if (update_g && D > 1) {
            T* G1 = sh.G + G.db[1];
            T g = G1[a];
            for (int n = 2; n <= D; ++n) g = fma(sh.num[n], chain(sg, sh.Tb, n, 1)[a], g);
            G1[a] = g;
        }
    }
    if (update_g && update_upper) {
        uint32_t u = threadIdx.x;
        for (int i = 2; i < D; ++i) {
            const uint32_t wi = G.pw[i];
            T* Gi = sh.G + G.db[i];
            for (; u < wi; u += blockDim.x) {
                T s = Gi[u];
                for (int n = i + 1; n <= D; ++n) s = fma(sh.num[n - i + 1], chain(sg, sh.Tb, n, i)[u], s);
                Gi[u] = s;
            }
            u -= wi;
        }
    }
}

// One reverse step for increment k.  `pending_grad` (non-null) = the previous
// reverse step still has to be finished (its gradient row); that runs inside
// the first recovery stage.  Ends with a barrier after which xc_next holds the
// increment of step k-1 and this step's partials are in sh.part.
template <typename T, int WT>
__device__ __forceinline__ void backward_step(const SigGeometry& sg, const SigShared<T>& sh, const T* xc,
                                              T* xc_next, T x_next, T* pending_grad) {
    const Geometry& G = sg.g;
    const Width<WT> Wd(G);
    const uint32_t W = Wd.value();
    const int D = G.depth;
    T* S = sh.S;
    const T s0 = S[0];
    const T* x1 = xc + W;
    const uint32_t slots = blockDim.x / W;
    const uint32_t my_a = threadIdx.x % W, my_slot = threadIdx.x / W;
    const bool xbar_lane = my_slot < slots;

    // Phase A: recover S_1..S_{D-1} of the prefix and the forward chains.
    if (D == 1 && pending_grad) {
        finish_reverse_step(sg, sh, pending_grad, true, partial_groups(W));
        __syncthreads();
    }
    for (int j = 1; j < D; ++j) {
        if (j == 1 && pending_grad) finish_reverse_step(sg, sh, pending_grad, true, partial_groups(W));
        const uint32_t wj = G.pw[j];
        T* Sj = S + G.db[j];
        const T* own = chain(sg, sh.Tf, j, j - 1);
        if constexpr (kRowModeA<WT>) {
            const uint32_t rows = G.pw[j - 1];
            if (rows >= kRowMin) {  // (so j >= 2 and every prefix comes from a chain)
                for (uint32_t q = threadIdx.x; q < rows; q += blockDim.x) {
                    const T o = own[q];
                    T* Sq = Sj + q * WT;
                    T s[WT];
#pragma unroll
                    for (int a = 0; a < WT; ++a) {
                        s[a] = fma(-o, x1[a], Sq[a]);
                        Sq[a] = s[a];
                    }
                    for (int n = j + 1; n <= D; ++n) {
                        const T p = chain(sg, sh.Tf, n, j - 1)[q];
                        const T* xm = xc + (n - j + 1) * WT;
                        T* dst = chain(sg, sh.Tf, n, j) + q * WT;
#pragma unroll
                        for (int a = 0; a < WT; ++a) dst[a] = fma(p, xm[a], s[a]);
                    }
                }
                __syncthreads();
                continue;
            }
        }
        for (uint32_t u = threadIdx.x; u < wj; u += blockDim.x) {
            uint32_t q, a;
            Wd.divmod(u, q, a);
            const T s = fma(-(j == 1 ? s0 : own[q]), x1[a], Sj[u]);
            Sj[u] = s;
            for (int n = j + 1; n <= D; ++n) {
                const T p = j == 1 ? s0 : chain(sg, sh.Tf, n, j - 1)[q];
                chain(sg, sh.Tf, n, j)[u] = fma(p, xc[(n - j + 1) * W + a], s);
            }
        }
        __syncthreads();
    }

    // Phase B: scaled cotangent chains, top stage first.  Letter gradients:
    // with kFusedLetters the thread that takes a row also adds
    // row[a] * T^n_{j-1}[r] to its accumulator of letter a (one read of the row
    // serves both sums); otherwise the xbar partials are letter-specialised:
    // thread t accumulates letter t % W only.
    T xacc = T(0);
    T xa[kFusedLetters<WT> ? WT : 1];
#pragma unroll
    for (int a = 0; a < (kFusedLetters<WT> ? WT : 1); ++a) xa[a] = T(0);
    for (int j = D; j >= 2; --j) {
        const uint32_t wjm1 = G.pw[j - 1];
        if constexpr (kFusedLetters<WT>) {
            // the chains of this stage as one run of rows (offsets carried
            // across chains), the scaled increment in registers
            uint32_t r = threadIdx.x;
            for (int n = j; n <= D; ++n) {
                if (r < wjm1) {
                    const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                    const T* tprev = chain(sg, sh.Tf, n, j - 1);
                    T* gout = chain(sg, sh.Tb, n, j - 1);
                    T x[WT];
                    load_row(x, xc + (n - j + 2) * WT);
                    for (; r < wjm1; r += blockDim.x) {
                        const T* row = gin + r * WT;
                        const T tp = tprev[r];
                        T acc = T(0);
#pragma unroll
                        for (int a = 0; a < WT; ++a) {
                            const T g = row[a];
                            acc = fma(g, x[a], acc);
                            xa[a] = fma(g, tp, xa[a]);
                        }
                        gout[r] = acc;
                    }
                }
                r -= wjm1;
            }
        } else {
            if constexpr (kRowModeB<WT>) {
                // the same run of rows, without the letter sums
                uint32_t r = threadIdx.x;
                for (int n = j; n <= D; ++n) {
                    if (r < wjm1) {
                        const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                        T* gout = chain(sg, sh.Tb, n, j - 1);
                        T x[WT];
                        load_row(x, xc + (n - j + 2) * WT);
                        for (; r < wjm1; r += blockDim.x) {
                            const T* row = gin + r * WT;
                            T acc = T(0);
#pragma unroll
                            for (int a = 0; a < WT; ++a) acc = fma(row[a], x[a], acc);
                            gout[r] = acc;
                        }
                    }
                    r -= wjm1;
                }
            } else {
                for (int n = j; n <= D; ++n) {
                    const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                    T* gout = chain(sg, sh.Tb, n, j - 1);
                    const T* xm = xc + (n - j + 2) * W;
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
            }
            if (xbar_lane) {
                // rows of all chains of the stage in one run (offsets carried)
                uint32_t u = my_slot;
                for (int n = j; n <= D; ++n) {
                    const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                    const T* tprev = chain(sg, sh.Tf, n, j - 1);
#pragma unroll 4
                    for (; u < wjm1; u += slots) xacc = fma(gin[u * W + my_a], tprev[u], xacc);
                    u -= wjm1;
                }
            }
        }
        __syncthreads();
    }
    if constexpr (kFusedLetters<WT>)
        store_letter_partials<T, WT>(sh, xa);
    else
        store_partials(sh, xbar_lane ? xacc : T(0), W);
    set_increment(sg, sh, xc_next, x_next);
    __syncthreads();
}

// One reverse step with D barriers instead of 2D - 1.  The recovery of the
// prefix (phase A, bottom-up) and the transposition of the cotangent chains
// (phase B, top-down) touch disjoint arrays -- A reads and writes S and the
// forward chains Tf, B reads G and the cotangent chains Tb and writes Tb --
// so stage s (s = 1..D-1) runs A's level s beside B's level D+1-s.  Phase B's
// letter gradients need every forward chain link, so they move to one last
// stage, together with the update of G's levels 2..D-1; there each
// coefficient (u, a) of a level is owned by one thread, which reads its old
// G value (for the letter sum) before writing the updated one, so no barrier
// separates the two.  G_1 and the gradient row are finished in the next
// step's first stage by the gradient lanes, as in backward_step.  The sums are
// the same as backward_step's in a different order.
template <typename T, int WT>
__device__ __forceinline__ void backward_step_merged(const SigGeometry& sg, const SigShared<T>& sh, const T* xc,
                                                     T* xc_next, T x_next, T* pending_grad) {
    const Geometry& G = sg.g;
    const Width<WT> Wd(G);
    const uint32_t W = Wd.value();
    const int D = G.depth;
    T* S = sh.S;
    const T s0 = S[0];
    const T* x1 = xc + W;
    const uint32_t bd = blockDim.x;

    // With D <= 2 stage 1's transposition overwrites Tb^D_1, which finishing
    // the previous step reads: finish it in a stage of its own.
    if (D <= 2 && pending_grad) {
        finish_reverse_step(sg, sh, pending_grad, true, partial_groups(W), false);
        __syncthreads();
        pending_grad = nullptr;
    }
    for (int st = 1; st < D; ++st) {
        if (st == 1 && pending_grad) finish_reverse_step(sg, sh, pending_grad, true, partial_groups(W), false);
        uint32_t r = threadIdx.x;
        // A: recover S_st of the prefix and the chain links T^n_st, n > st
        {
            const int j = st;
            const uint32_t wj = G.pw[j];
            T* Sj = S + G.db[j];
            const T* own = chain(sg, sh.Tf, j, j - 1);
            bool done = false;
            if constexpr (kRowModeA<WT>) {
                const uint32_t rows = G.pw[j - 1];
                if (rows >= kRowMin) {
                    for (; r < rows; r += bd) {
                        const T o = own[r];
                        T* Sq = Sj + r * WT;
                        T sv[WT];
#pragma unroll
                        for (int a = 0; a < WT; ++a) {
                            sv[a] = fma(-o, x1[a], Sq[a]);
                            Sq[a] = sv[a];
                        }
                        for (int n = j + 1; n <= D; ++n) {
                            const T p = chain(sg, sh.Tf, n, j - 1)[r];
                            const T* xm = xc + (n - j + 1) * WT;
                            T* dst = chain(sg, sh.Tf, n, j) + r * WT;
#pragma unroll
                            for (int a = 0; a < WT; ++a) dst[a] = fma(p, xm[a], sv[a]);
                        }
                    }
                    r -= rows;
                    done = true;
                }
            }
            if (!done) {
                for (; r < wj; r += bd) {
                    uint32_t q, a;
                    Wd.divmod(r, q, a);
                    const T sv = fma(-(j == 1 ? s0 : own[q]), x1[a], Sj[r]);
                    Sj[r] = sv;
                    for (int n = j + 1; n <= D; ++n) {
                        const T p = j == 1 ? s0 : chain(sg, sh.Tf, n, j - 1)[q];
                        chain(sg, sh.Tf, n, j)[r] = fma(p, xc[(n - j + 1) * W + a], sv);
                    }
                }
                r -= wj;
            }
        }
        // B: the cotangent chains n = j..D from level j to level j - 1, j = D + 1 - st
        {
            const int j = D + 1 - st;
            const uint32_t wjm1 = G.pw[j - 1];
            for (int n = j; n <= D; ++n) {
                if (r < wjm1) {
                    const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                    T* gout = chain(sg, sh.Tb, n, j - 1);
                    if constexpr (kRowModeB<WT>) {
                        T x[WT];
                        load_row(x, xc + (n - j + 2) * WT);
                        for (; r < wjm1; r += bd) {
                            const T* row = gin + r * WT;
                            T acc = T(0);
#pragma unroll
                            for (int a = 0; a < WT; ++a) acc = fma(row[a], x[a], acc);
                            gout[r] = acc;
                        }
                    } else {
                        const T* xm = xc + (n - j + 2) * W;
                        for (; r < wjm1; r += bd) {
                            const T* row = gin + r * W;
                            T acc = T(0);
                            if constexpr (WT > 0) {
#pragma unroll
                                for (int a = 0; a < WT; ++a) acc = fma(row[a], xm[a], acc);
                            } else {
                                for (uint32_t a = 0; a < W; ++a) acc = fma(row[a], xm[a], acc);
                            }
                            gout[r] = acc;
                        }
                    }
                }
                r -= wjm1;
            }
        }
        __syncthreads();
    }

    // Letter gradients of levels 2..D and the update of G_2..G_{D-1}.  Thread
    // t takes letter t mod W of rows t / W, t / W + slots, ... (one run over
    // the levels, offsets carried).
    const uint32_t slots = bd / W;
    const uint32_t my_a = threadIdx.x % W, my_slot = threadIdx.x / W;
    T xacc = T(0);
    if (my_slot < slots) {
        uint32_t u = my_slot;
        for (int j = 2; j <= D; ++j) {
            const uint32_t rows = G.pw[j - 1];
            T* Gj = j == D ? sh.top : sh.G + G.db[j];
            for (; u < rows; u += slots) {
                const uint32_t idx = u * W + my_a;
                const T g = Gj[idx];
                xacc = fma(g, chain(sg, sh.Tf, j, j - 1)[u], xacc);
                T gn = g;
                for (int n = j + 1; n <= D; ++n) {
                    const T t = chain(sg, sh.Tb, n, j)[idx];
                    xacc = fma(t, chain(sg, sh.Tf, n, j - 1)[u], xacc);
                    gn = fma(sh.num[n - j + 1], t, gn);
                }
                if (j < D) Gj[idx] = gn;
            }
            u -= rows;
        }
    }
    store_partials(sh, my_slot < slots ? xacc : T(0), W);
    set_increment(sg, sh, xc_next, x_next);
    __syncthreads();
}

// Kernel body.  With `gws` null every array lives in shared memory; otherwise
// the state and chain arrays of CTA i live in gws + i*gws_stride (global
// memory, L2-resident at the grid sizes used) and only the increments,
// 1/m and the partials stay in shared memory.
// Registers: at most 64 per thread for FP64 (two 512-thread blocks per SM;
// the fastest measured), 40 for FP32, whose small states fit more CTAs per SM
// than 64 registers allow (ragged W8 D4 FP32: 29.3 -> 28.3 ms).
// COT: the cotangent arrays may live in the global workspace (kCotGlobal) --
// a separate instantiation, so that the other kernels' code is what it was
// without that option (it cost W16 D3 2.6 % when it was a run-time choice).
template <typename T, int WT, int MAXT, bool COT = false>
__global__ void __launch_bounds__(MAXT, (MAXT <= 512 ? (sizeof(T) == 4 ? 3 : 2) : 1)) k_signature(SigGeometry sg, const T* __restrict__ incr, PathBatch paths,
                                                    T* sig, int64_t sig_stride, const T* seed, int64_t seed_stride,
                                                    T* grad, int mode, T* gws, int64_t gws_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t dim = G.dim;
    const uint32_t lo = G.db[D];  // coefficients below the top level
    const bool bwd = mode & kBackward;
    const bool fwd_top = mode & kTopLevel;
    const bool top_global = mode & kTopGlobal;
    const uint32_t held = top_global ? lo : dim;  // coefficients of S kept on chip
    const int nmax = fwd_top ? D : D - 1;

    SigShared<T> sh;
    T* q = reinterpret_cast<T*>(smem_raw);
    // kCotGlobal: S and the forward chains in shared memory, the cotangent
    // level and chains in this CTA's slice of the global workspace
    const bool cot_global = COT && (mode & kCotGlobal) && bwd && gws;
    T* p = (gws && !cot_global) ? gws + blockIdx.x * gws_stride : q;
    // the FP32 four-coefficient forward step wants S + 1, Tf + choff[1] and the
    // scaled increments on 16-byte boundaries (kVec4; the host adds slack)
    bool vec4 = false;
    if constexpr (kVec4<T, WT>) vec4 = gws == nullptr && !top_global;
    auto align4 = [&](uint32_t off) {  // elements to skip so that p + off is 16-byte aligned
        return vec4 ? static_cast<uint32_t>((4u - (static_cast<uint32_t>(p - q) + off) % 4u) % 4u) : 0u;
    };
    p += align4(1);
    sh.S = p;
    sh.top = p + lo;
    p += held;
    p += align4(sg.choff[1]);
    sh.Tf = p;
    p += sg.chain_total;
    if (bwd) {
        T* g = cot_global ? gws + blockIdx.x * gws_stride : p;
        sh.G = g;
        g += lo;
        sh.Tb = g;
        g += sg.chain_total;
        if (!cot_global) p = g;
    } else {
        sh.G = sh.Tb = nullptr;
    }
    if (gws && !cot_global) p = q;
    p += align4(0);
    sh.xcs = (D + 1) * W;
    sh.xc = p;
    p += 2 * sh.xcs;
    sh.inv = p;
    p += D + 1;
    sh.num = p;
    p += D + 2;
    sh.part = p;
    for (int m = threadIdx.x; m <= D; m += blockDim.x) sh.inv[m] = m == 0 ? T(0) : T(1) / static_cast<T>(m);
    for (int m = threadIdx.x; m <= D + 1; m += blockDim.x) sh.num[m] = static_cast<T>(m);
    __syncthreads();

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
        const T* xin = incr + off * W;

        if (mode & kLoadFinal) {
            const T* src = sig + b * sig_stride;
            for (uint32_t i = threadIdx.x; i < lo; i += blockDim.x) sh.S[i] = src[i];
        } else {
            for (uint32_t i = threadIdx.x; i < held; i += blockDim.x) sh.S[i] = i == 0 ? T(1) : T(0);
            if (top_global && fwd_top) {
                sh.top = sig + b * sig_stride + lo;
                for (uint32_t i = threadIdx.x; i < G.pw[D]; i += blockDim.x) sh.top[i] = T(0);
            }
        }

        if (mode & kForward) {
            if (len > 0) set_increment(sg, sh, xc_buf(sh, 0), load_increment(sg, xin, 0));
            __syncthreads();
            T xv = len > 1 ? load_increment(sg, xin, 1) : T(0);
            for (int64_t k = 0; k < len; ++k) {
                const T x_next = xv;
                if (k + 2 < len) xv = load_increment(sg, xin, k + 2);
                forward_step<T, WT>(sg, sh, xc_buf(sh, k), xc_buf(sh, k + 1), x_next, nmax, top_global, vec4);
            }
            if (sig && !(mode & kLoadFinal)) {
                T* dst = sig + b * sig_stride;
                for (uint32_t i = threadIdx.x; i < held; i += blockDim.x) dst[i] = sh.S[i];
            }
            __syncthreads();
        }
        if (bwd) {
            const T* sd = seed + b * seed_stride;
            for (uint32_t i = threadIdx.x; i < lo; i += blockDim.x) sh.G[i] = sd[i];
            if (top_global)
                sh.top = const_cast<T*>(sd) + lo;  // read only in the reverse pass
            else
                for (uint32_t i = threadIdx.x; i < G.pw[D]; i += blockDim.x) sh.top[i] = sd[lo + i];
            T* gout = grad + off * W;
            if (len > 0) set_increment(sg, sh, xc_buf(sh, len - 1), load_increment(sg, xin, len - 1));
            __syncthreads();
            T xv = len > 1 ? load_increment(sg, xin, len - 2) : T(0);
            for (int64_t k = len - 1; k >= 0; --k) {
                const T x_next = xv;
                if (k >= 2) xv = load_increment(sg, xin, k - 2);
                if (mode & kMergedReverse)
                    backward_step_merged<T, WT>(sg, sh, xc_buf(sh, k), xc_buf(sh, k - 1), x_next,
                                                k + 1 < len ? gout + (k + 1) * W : nullptr);
                else
                    backward_step<T, WT>(sg, sh, xc_buf(sh, k), xc_buf(sh, k - 1), x_next,
                                         k + 1 < len ? gout + (k + 1) * W : nullptr);
            }
            if (len > 0) {
                finish_reverse_step(sg, sh, gout, false, partial_groups(W));
                __syncthreads();
            }
        }
        __syncthreads();
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
constexpr int kLengthBuckets = 4 * 40;

__device__ __forceinline__ int length_bucket(int64_t len) {
    if (len <= 0) return 0;
    const int msb = 63 - __clzll(static_cast<unsigned long long>(len));
    const int sub = msb >= 2 ? static_cast<int>((len >> (msb - 2)) & 3) : static_cast<int>((len << (2 - msb)) & 3);
    const int key = 1 + msb * 4 + sub;
    return key < kLengthBuckets ? key : kLengthBuckets - 1;
}

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

// Elements of the state and chain arrays of one CTA (without the top level
// when it lives in global memory).
size_t sig_state_elems(const SigGeometry& sg, bool bwd, bool top_global = false) {
    size_t n = (top_global ? sg.g.db[sg.g.depth] : sg.g.dim) + sg.chain_total;
    if (bwd) n += sg.g.db[sg.g.depth] + sg.chain_total;
    return n;
}

// Shared memory of one CTA: the small arrays, plus the state when resident.
template <typename T>
size_t sig_smem_bytes(const SigGeometry& sg, int threads, bool bwd, bool resident, bool top_global = false) {
    const size_t D = sg.g.depth, W = sg.g.width;
    size_t n = 2 * (D + 1) * W + (D + 1) + (D + 2) + threads;
    if (resident) n += sig_state_elems(sg, bwd, top_global);
    if (std::is_same<T, float>::value) n += 12;  // alignment padding of the FP32 four-coefficient step
    return n * sizeof(T);
}

// Threads per CTA of the global-workspace variant (one CTA per SM), and the
// largest CTA the shared-memory variant may be tuned to.
constexpr int kWideThreads = 1024;
constexpr int kResidentMaxThreads = 512;

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

SigLaunches plan_launches(bool forward, bool has_sig, bool has_seed, bool has_grad, int threads) {
    SigLaunches l;
    const bool split = forward && has_sig && has_seed && has_grad && threads > 0 && (threads & kScheduleSplit);
    if (split) {
        const bool fwd_top_global = threads & kScheduleForwardTopGlobal;
        const int rev = (threads >> kScheduleReverseShift) & 1023;
        const int cot = threads & (kScheduleCotangentGlobal | kScheduleMergedReverse);
        const int fwd = threads & ((1 << 14) - 1);  // CTA size and cap
        l.count = 2;
        l.mode[0] = kForward | kTopLevel | (fwd_top_global ? kTopGlobal : 0);
        l.schedule[0] = fwd;
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
    l.count = 1;
    l.mode[0] = mode;
    l.schedule[0] = threads;
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
    const SigLaunches launches = plan_launches(forward, sig != nullptr, seed != nullptr, grad != nullptr, threads);
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
    const SigLaunches launches = plan_launches(true, sig != nullptr, seed != nullptr, grad != nullptr, threads);
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
