// signature_body.cuh -- the per-path device code of the fused signature
// kernels (signature.cu: k_signature; signature_group.cu: the grouped launch).
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
#pragma once

#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "launch_util.cuh"
#include "ops.hpp"

namespace rpp_gb {
namespace {


// Threads per CTA of the global-workspace variant (one CTA per SM), and the
// largest CTA the shared-memory variant may be tuned to.
constexpr int kWideThreads = 1024;
constexpr int kResidentMaxThreads = 512;

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
// kTopRegs (FP32 forward-only, TOPROWS > 0): the top level in registers, each
// thread holding whole rows of W coefficients for the whole path (no chain
// reads the top level, so no other thread needs it); see forward_step.
enum SigMode : int {
    kForward = 1,
    kBackward = 2,
    kLoadFinal = 4,
    kTopLevel = 8,
    kTopGlobal = 16,
    kCotGlobal = 32,
    kMergedReverse = 64,
    kTopRegs = 128
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
    // Letter of the first level-1 coefficient held: 0, except in a CTA of a
    // cluster that splits a path's state by first letter (k_signature_split),
    // whose level-1 slice holds letters lofs .. lofs + W/P - 1.
    uint32_t lofs;
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

// The threads that run one path.  CtaTeam: the whole CTA (barrier 0).
// SubTeam: `n` consecutive threads starting at a multiple of 32, with a
// named barrier of their own (bar.sync id, n; ids 1..15), so that one CTA of
// the grouped launch runs several small paths side by side.  Every device
// function below takes its thread rank, thread count and barrier from the
// team.
struct CtaTeam {
    __device__ __forceinline__ uint32_t rank() const { return threadIdx.x; }
    __device__ __forceinline__ uint32_t size() const { return blockDim.x; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
};

struct SubTeam {
    uint32_t r;   // rank inside the team
    uint32_t n;   // threads of the team (a multiple of 32)
    uint32_t id;  // named barrier
    __device__ __forceinline__ uint32_t rank() const { return r; }
    __device__ __forceinline__ uint32_t size() const { return n; }
    __device__ __forceinline__ void sync() const { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
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
template <typename T, typename Team>
__device__ __forceinline__ void set_increment(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh, T* xc, T xv) {
    const uint32_t W = static_cast<uint32_t>(sg.g.width);
    const uint32_t t = tm.rank();
    if (t < static_cast<uint32_t>(sg.g.depth) * W) {
        const uint32_t m = 1 + t / W;
        xc[m * W + t % W] = xv * sh.inv[m];
    }
}

template <typename T, typename Team>
__device__ __forceinline__ T load_increment(const Team& tm, const SigGeometry& sg, const T* path_incr, int64_t k) {
    const uint32_t W = static_cast<uint32_t>(sg.g.width);
    const uint32_t t = tm.rank();
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
// Rows of the top level a thread keeps in registers with kTopRegs (32
// registers of state: 8 rows at W = 4, 4 at W = 8, 2 at W = 16).
template <typename T, int WT>
constexpr int kTopRows = kVec4<T, WT> ? 32 / WT : 0;

template <typename T, int WT>
using TopRegs = T[kTopRows<T, WT> > 0 ? kTopRows<T, WT> : 1][WT > 0 ? WT : 1];

// TOPREGS (FP32, W a multiple of 4, the top level maintained, D >= 2): the
// last stage updates levels 1..D-1 in shared memory and the top level in
// `top`: thread t holds rows t, t + n, ... (n threads) -- W coefficients
// sharing the prefix T^D_{D-1}[row] -- so one shared load serves W FMAs with
// the increment in registers, where the shared-memory form loads and stores
// the state and the increment for every four FMAs.
template <typename T, int WT, bool SPLIT = false, bool TOPREGS = false, typename Team = CtaTeam>
__device__ __forceinline__ void forward_step(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh, const T* xc,
                                             T* xc_next, T x_next, int nmax, bool top_global, bool vec4,
                                             TopRegs<T, WT>* top = nullptr) {
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
                uint32_t v = tm.rank();  // groups of four coefficients
                for (int n = j + 1; n <= nmax; ++n) {
                    const T* prev = chain(sg, sh.Tf, n, j - 1);
                    float4* dst = reinterpret_cast<float4*>(chain(sg, sh.Tf, n, j));
                    const T* xm = xc + (n - j + 1) * WT;
                    const uint32_t groups = wj / 4;
                    for (; v < groups; v += tm.size()) {
                        const uint32_t u = 4 * v, q = u / WT, a = u % WT;
                        const T pq = j == 1 ? s0 : prev[q];
                        const float4 sv = reinterpret_cast<const float4*>(Sj)[v];
                        const float4 xv = *reinterpret_cast<const float4*>(xm + a);
                        dst[v] = make_float4(fmaf(pq, xv.x, sv.x), fmaf(pq, xv.y, sv.y), fmaf(pq, xv.z, sv.z),
                                             fmaf(pq, xv.w, sv.w));
                    }
                    v -= groups;
                }
                tm.sync();
                continue;
            }
        }
        uint32_t u = tm.rank();
        for (int n = j + 1; n <= nmax; ++n) {
            T* dst = chain(sg, sh.Tf, n, j);
            const T* prev = chain(sg, sh.Tf, n, j - 1);
            const T* xm = xc + (n - j + 1) * W;
            for (; u < wj; u += tm.size()) {
                uint32_t q, a;
                Wd.divmod(u, q, a);
                if constexpr (SPLIT) a += j == 1 ? sh.lofs : 0u;
                const T p = j == 1 ? s0 : prev[q];
                dst[u] = fma(p, xm[a], Sj[u]);
            }
            u -= wj;
        }
        tm.sync();
    }
    const T* x1 = xc + W;
    int n_first = 1;
    if constexpr (kVec4<T, WT>) {
        if (vec4) {  // (top level in shared memory, or in registers)
            uint32_t v = tm.rank();
            for (int n = 1; n <= (TOPREGS ? nmax - 1 : nmax); ++n) {
                const T* prev = chain(sg, sh.Tf, n, n - 1);
                float4* Sn = reinterpret_cast<float4*>(S + G.db[n]);
                const uint32_t groups = G.pw[n] / 4;
                for (; v < groups; v += tm.size()) {
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
            if constexpr (TOPREGS && kTopRows<T, WT> > 0) {
                const int D = G.depth;
                const T* prev = chain(sg, sh.Tf, D, D - 1);
                T xr[WT];
#pragma unroll
                for (int a = 0; a < WT; a += 4) {
                    const float4 xv = *reinterpret_cast<const float4*>(x1 + a);
                    xr[a] = xv.x;
                    xr[a + 1] = xv.y;
                    xr[a + 2] = xv.z;
                    xr[a + 3] = xv.w;
                }
#pragma unroll
                for (int i = 0; i < kTopRows<T, WT>; ++i) {
                    const uint32_t r = tm.rank() + i * tm.size();
                    if (r < G.pw[D - 1]) {
                        const T p = prev[r];
#pragma unroll
                        for (int a = 0; a < WT; ++a) (*top)[i][a] = fmaf(p, xr[a], (*top)[i][a]);
                    }
                }
            }
        }
    }
    uint32_t v = tm.rank();
    for (int n = n_first; n <= nmax; ++n) {
        const uint32_t wn = G.pw[n];
        T* Sn = n == G.depth ? sh.top : S + G.db[n];
        const T* prev = chain(sg, sh.Tf, n, n - 1);
        if (n == G.depth && top_global) {
            // S_D in global memory: four independent read-modify-writes per
            // batch, so their L2 latencies overlap (each coefficient is owned
            // by one thread for the whole path)
            const uint32_t bd = tm.size();
            for (uint32_t u0 = tm.rank(); u0 < wn; u0 += 4 * bd) {
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
                        if constexpr (SPLIT) a += n == 1 ? sh.lofs : 0u;
                        Sn[u] = fma(n == 1 ? s0 : prev[q], x1[a], v[k]);
                    }
                }
            }
            continue;
        }
        for (; v < wn; v += tm.size()) {
            uint32_t q, a;
            Wd.divmod(v, q, a);
            if constexpr (SPLIT) a += n == 1 ? sh.lofs : 0u;
            const T p = n == 1 ? s0 : prev[q];
            Sn[v] = fma(p, x1[a], Sn[v]);
        }
        v -= wn;
    }
    set_increment(tm, sg, sh, xc_next, x_next);
    tm.sync();
}

// Partial letter gradients of one reverse step.  Thread t accumulated letter
// t mod W; lanes of a warp with the same letter (lanes l, l + W, l + 2W, ...)
// are summed by a shuffle tree, and lane l < W of warp w stores the warp's
// partial of letter (32w + l) mod W at part[w*W + letter] -- log2(32/W) adds
// per warp instead of W threads each adding blockDim/W partials in sequence.
// W > 16 keeps one partial per thread (part[t]).  partial_groups() gives the
// number of partials per letter either way.
template <typename T, typename Team>
__device__ __forceinline__ void store_partials(const Team& tm, const SigShared<T>& sh, T v, uint32_t W) {
    if (W > 16) {
        sh.part[tm.rank()] = v;
        return;
    }
    const uint32_t lane = tm.rank() & 31u;
    for (uint32_t off = W; off < 32u; off *= 2u) {
        const T o = __shfl_down_sync(0xffffffffu, v, off);
        if (lane + off < 32u) v += o;
    }
    if (lane < W) sh.part[(tm.rank() >> 5) * W + tm.rank() % W] = v;
}

template <typename Team>
__device__ __forceinline__ uint32_t partial_groups(const Team& tm, uint32_t W) { return W > 16 ? tm.size() / W : tm.size() / 32; }

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

template <typename T, int WT, typename Team>
__device__ __forceinline__ void store_letter_partials(const Team& tm, const SigShared<T>& sh, T (&xa)[WT]) {
    const uint32_t lane = tm.rank() & 31u;
    uint32_t base = 0, cnt = WT;
    letter_butterfly<T, WT>(xa, lane, 16u, base, cnt);
    // lanes that differ only in the bits of the plain xor levels hold the same
    // total; the one with those bits zero stores it
    constexpr uint32_t halvings = WT <= 1 ? 0u : WT <= 2 ? 1u : WT <= 4 ? 2u : WT <= 8 ? 3u : 4u;
    if (cnt > 0u && (lane & ((32u >> halvings) - 1u)) == 0u)
        sh.part[(tm.rank() >> 5) * WT + base] = xa[0];
}

// G_{k-1,i} = G_i + sum_{n>i} (n-i+1) Gh^n_i for the levels i = 2..D-1, as
// one run of coefficients over all threads.
template <typename T, typename Team>
__device__ __forceinline__ void update_upper_g(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    uint32_t u = tm.rank();
    for (int i = 2; i < D; ++i) {
        const uint32_t wi = G.pw[i];
        T* Gi = sh.G + G.db[i];
        for (; u < wi; u += tm.size()) {
            T s = Gi[u];
            for (int n = i + 1; n <= D; ++n) s = fma(sh.num[n - i + 1], chain(sg, sh.Tb, n, i)[u], s);
            Gi[u] = s;
        }
        u -= wi;
    }
}

// Finish a reverse step: grad_k from the partials (the stage-1 terms
// sum_n Gh^n_1[a] S_0 folded in) and, when `update_g`, G_{k-1} from the
// cotangent chains.  Runs between barriers, beside the first recovery stage,
// which runs on warp 0: the W gradient lanes are the first W threads of the
// CTA's last warp(s), and each of them updates G_1[a] after reading it.  The
// other levels of G form one run of coefficients over all threads.
template <typename T, typename Team>
__device__ __forceinline__ void finish_reverse_step(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh, T* grad_k,
                                                    bool update_g, uint32_t groups, bool update_upper = true) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const T s0 = sh.S[0];
    const uint32_t gl = tm.size() - ((W + 31u) & ~31u);  // (team size >= W, both multiples of 32 after rounding)
    if (tm.rank() >= gl && tm.rank() < gl + W) {
        const uint32_t a = tm.rank() - gl;
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
    if (update_g && update_upper) update_upper_g(tm, sg, sh);
}

// Split state (k_signature_split): a cluster of P CTAs holds one path, CTA
// `rank` the coefficients of every level j >= 1 whose first letter lies in
// [rank W/P, (rank+1) W/P) -- W^j / P consecutive coefficients of level j.
// A coefficient's Horner parent is its prefix, which has the same first
// letter, so every chain link, the recovery of the prefix and the
// transposition of the cotangent chains stay inside one CTA; the kernel runs
// the single-CTA code on the sliced geometry, with level-1 letters offset by
// lofs.  Only the letter gradients cross CTAs: xbar_a sums over all words
// ending in a, whatever their first letter.  Each CTA adds up its own words'
// terms per letter and stores them in rank 0's shared memory
// (slots[step parity][rank][letter], distributed shared memory); rank 0 adds
// the P partials in rank order and writes the gradient row.
template <typename T>
struct SplitCtx {
    T* slots;       // this CTA's [2][P][W] exchange buffer (rank 0's is read)
    uint32_t P;
    uint32_t rank;
    T* gout;        // the path's gradient rows
    int64_t len;    // the path's increments
};

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Stores v at `local` (an address in this CTA's shared memory) in the shared
// memory of cluster CTA `rank` (same layout).
template <typename T>
__device__ __forceinline__ void store_remote(T* local, uint32_t rank, T v) {
    const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(local));
    uint32_t remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(addr), "r"(rank));
    static_assert(sizeof(T) == 8 || sizeof(T) == 4, "8- or 4-byte values");
    if constexpr (sizeof(T) == 8) {
        unsigned long long bits;
        memcpy(&bits, &v, 8);
        asm volatile("st.shared::cluster.b64 [%0], %1;" ::"r"(remote), "l"(bits) : "memory");
    } else {
        unsigned int bits;
        memcpy(&bits, &v, 4);
        asm volatile("st.shared::cluster.b32 [%0], %1;" ::"r"(remote), "r"(bits) : "memory");
    }
}

// The exchange of the partials of reverse step m (run in step m-1's first
// stage, or after the last step for m = 0), by every thread of the CTA:
// (a) unless m is the path's last increment, wait on the cluster barrier,
// after which every CTA's partials of step m+1 are in rank 0's slots, and
// rank 0's gradient lanes write gradient row m+1 (the P partials added in
// rank order); (b) the gradient lanes form this CTA's partial of step m --
// its partial groups, plus for the letters it owns the stage-1 terms
// sum_n Gh^n_1[a] S_0 -- and store it in rank 0's slots; the owners update
// G_1 and, with `update_g`, all threads G's levels 2..D-1 (as
// finish_reverse_step); (c) arrive on the cluster barrier.  Slots of one
// parity are rewritten two steps later, after the wait that follows rank 0's
// reads of them.
template <typename T, typename Team>
__device__ __forceinline__ void split_exchange(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh,
                                               const SplitCtx<T>& cx, int64_t m, bool update_g) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t per = W / cx.P;
    if (m + 1 < cx.len) cluster_wait();
    const uint32_t gl = tm.size() - ((W + 31u) & ~31u);
    if (tm.rank() >= gl && tm.rank() < gl + W) {
        const uint32_t a = tm.rank() - gl;
        const bool own = a >= sh.lofs && a < sh.lofs + per;
        if (cx.rank == 0 && m + 1 < cx.len) {
            const T* sl = cx.slots + ((m + 1) & 1) * cx.P * W;
            T v = T(0);
            for (uint32_t r = 0; r < cx.P; ++r) v += sl[r * W + a];
            cx.gout[(m + 1) * W + a] = v;
        }
        const T s0 = sh.S[0];
        T v = T(0);
        if (own) {
            const uint32_t la = a - sh.lofs;
            for (int n = 1; n <= D; ++n) {
                const T* g1 = n == 1 ? sh.G + G.db[1] : chain(sg, sh.Tb, n, 1);
                v = fma(g1[la], s0, v);
            }
        }
        const uint32_t groups = partial_groups(tm, W);
        for (uint32_t s = 0; s < groups; ++s) v += sh.part[s * W + a];
        store_remote(cx.slots + (m & 1) * cx.P * W + cx.rank * W + a, 0u, v);
        if (own && update_g) {
            T* G1 = sh.G + G.db[1];
            const uint32_t la = a - sh.lofs;
            T g = G1[la];
            for (int n = 2; n <= D; ++n) g = fma(sh.num[n], chain(sg, sh.Tb, n, 1)[la], g);
            G1[la] = g;
        }
    }
    if (update_g) update_upper_g(tm, sg, sh);
    cluster_arrive();
}

// After a path's last reverse step: the exchange of step 0, then rank 0
// writes gradient row 0.  Ends with a barrier of the CTA.
template <typename T, typename Team>
__device__ __forceinline__ void split_finish(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh,
                                             const SplitCtx<T>& cx) {
    const uint32_t W = static_cast<uint32_t>(sg.g.width);
    split_exchange(tm, sg, sh, cx, 0, false);
    cluster_wait();
    const uint32_t gl = tm.size() - ((W + 31u) & ~31u);
    if (cx.rank == 0 && tm.rank() >= gl && tm.rank() < gl + W) {
        const uint32_t a = tm.rank() - gl;
        T v = T(0);
        for (uint32_t r = 0; r < cx.P; ++r) v += cx.slots[r * W + a];
        cx.gout[a] = v;
    }
    tm.sync();
}

// One reverse step for increment k.  `pending_grad` (non-null) = the previous
// reverse step still has to be finished (its gradient row); that runs inside
// the first recovery stage.  Ends with a barrier after which xc_next holds the
// increment of step k-1 and this step's partials are in sh.part.
// SPLIT: one CTA of a split-state cluster; `sx` and `k` serve the exchange
// of the pending partials (those of step k+1) in place of finishing them.
template <typename T, int WT, bool SPLIT = false, typename Team = CtaTeam>
__device__ __forceinline__ void backward_step(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh, const T* xc,
                                              T* xc_next, T x_next, T* pending_grad,
                                              const SplitCtx<T>* sx = nullptr, int64_t k = 0) {
    const Geometry& G = sg.g;
    const Width<WT> Wd(G);
    const uint32_t W = Wd.value();
    const int D = G.depth;
    T* S = sh.S;
    const T s0 = S[0];
    const T* x1 = xc + W;
    const uint32_t slots = tm.size() / W;
    const uint32_t my_a = tm.rank() % W, my_slot = tm.rank() / W;
    const bool xbar_lane = my_slot < slots;

    // Phase A: recover S_1..S_{D-1} of the prefix and the forward chains.
    if (D == 1 && pending_grad) {
        finish_reverse_step(tm, sg, sh, pending_grad, true, partial_groups(tm, W));
        tm.sync();
    }
    for (int j = 1; j < D; ++j) {
        if constexpr (SPLIT) {
            if (j == 1 && pending_grad) split_exchange(tm, sg, sh, *sx, k + 1, true);
        } else {
            if (j == 1 && pending_grad) finish_reverse_step(tm, sg, sh, pending_grad, true, partial_groups(tm, W));
        }
        const uint32_t wj = G.pw[j];
        T* Sj = S + G.db[j];
        const T* own = chain(sg, sh.Tf, j, j - 1);
        if constexpr (kRowModeA<WT>) {
            const uint32_t rows = G.pw[j - 1];
            if (rows >= kRowMin) {  // (so j >= 2 and every prefix comes from a chain)
                for (uint32_t q = tm.rank(); q < rows; q += tm.size()) {
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
                tm.sync();
                continue;
            }
        }
        for (uint32_t u = tm.rank(); u < wj; u += tm.size()) {
            uint32_t q, a;
            Wd.divmod(u, q, a);
            if constexpr (SPLIT) a += j == 1 ? sh.lofs : 0u;
            const T s = fma(-(j == 1 ? s0 : own[q]), x1[a], Sj[u]);
            Sj[u] = s;
            for (int n = j + 1; n <= D; ++n) {
                const T p = j == 1 ? s0 : chain(sg, sh.Tf, n, j - 1)[q];
                chain(sg, sh.Tf, n, j)[u] = fma(p, xc[(n - j + 1) * W + a], s);
            }
        }
        tm.sync();
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
            uint32_t r = tm.rank();
            for (int n = j; n <= D; ++n) {
                if (r < wjm1) {
                    const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                    const T* tprev = chain(sg, sh.Tf, n, j - 1);
                    T* gout = chain(sg, sh.Tb, n, j - 1);
                    T x[WT];
                    load_row(x, xc + (n - j + 2) * WT);
                    for (; r < wjm1; r += tm.size()) {
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
                uint32_t r = tm.rank();
                for (int n = j; n <= D; ++n) {
                    if (r < wjm1) {
                        const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                        T* gout = chain(sg, sh.Tb, n, j - 1);
                        T x[WT];
                        load_row(x, xc + (n - j + 2) * WT);
                        // two rows per iteration, both rows' loads issued
                        // before either sum (the top stage's rows come from
                        // L2 when the seed's top level stays in global memory)
                        const uint32_t bd = tm.size();
                        for (; r + bd < wjm1; r += 2 * bd) {
                            T g0[WT], g1[WT];
                            load_row(g0, gin + r * WT);
                            load_row(g1, gin + (r + bd) * WT);
                            T acc0 = T(0), acc1 = T(0);
#pragma unroll
                            for (int a = 0; a < WT; ++a) {
                                acc0 = fma(g0[a], x[a], acc0);
                                acc1 = fma(g1[a], x[a], acc1);
                            }
                            gout[r] = acc0;
                            gout[r + bd] = acc1;
                        }
                        if (r < wjm1) {
                            const T* row = gin + r * WT;
                            T acc = T(0);
#pragma unroll
                            for (int a = 0; a < WT; ++a) acc = fma(row[a], x[a], acc);
                            gout[r] = acc;
                            r += bd;
                        }
                    }
                    r -= wjm1;
                }
            } else {
                for (int n = j; n <= D; ++n) {
                    const T* gin = n == j ? (j == D ? sh.top : sh.G + G.db[j]) : chain(sg, sh.Tb, n, j);
                    T* gout = chain(sg, sh.Tb, n, j - 1);
                    const T* xm = xc + (n - j + 2) * W;
                    for (uint32_t u = tm.rank(); u < wjm1; u += tm.size()) {
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
        tm.sync();
    }
    if constexpr (kFusedLetters<WT>)
        store_letter_partials<T, WT>(tm, sh, xa);
    else
        store_partials(tm, sh, xbar_lane ? xacc : T(0), W);
    set_increment(tm, sg, sh, xc_next, x_next);
    tm.sync();
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
template <typename T, int WT, typename Team>
__device__ __forceinline__ void backward_step_merged(const Team& tm, const SigGeometry& sg, const SigShared<T>& sh, const T* xc,
                                                     T* xc_next, T x_next, T* pending_grad) {
    const Geometry& G = sg.g;
    const Width<WT> Wd(G);
    const uint32_t W = Wd.value();
    const int D = G.depth;
    T* S = sh.S;
    const T s0 = S[0];
    const T* x1 = xc + W;
    const uint32_t bd = tm.size();

    // With D <= 2 stage 1's transposition overwrites Tb^D_1, which finishing
    // the previous step reads: finish it in a stage of its own.
    if (D <= 2 && pending_grad) {
        finish_reverse_step(tm, sg, sh, pending_grad, true, partial_groups(tm, W), false);
        tm.sync();
        pending_grad = nullptr;
    }
    for (int st = 1; st < D; ++st) {
        if (st == 1 && pending_grad) finish_reverse_step(tm, sg, sh, pending_grad, true, partial_groups(tm, W), false);
        uint32_t r = tm.rank();
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
        tm.sync();
    }

    // Letter gradients of levels 2..D and the update of G_2..G_{D-1}.  Thread
    // t takes letter t mod W of rows t / W, t / W + slots, ... (one run over
    // the levels, offsets carried).
    const uint32_t slots = bd / W;
    const uint32_t my_a = tm.rank() % W, my_slot = tm.rank() / W;
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
    store_partials(tm, sh, my_slot < slots ? xacc : T(0), W);
    set_increment(tm, sg, sh, xc_next, x_next);
    tm.sync();
}

// Placement of one CTA's arrays.  With `gws` null every array lives in shared
// memory; otherwise the state and chain arrays of CTA i live in
// gws + i*gws_stride (global memory, L2-resident at the grid sizes used) and
// only the increments, 1/m and the partials stay in shared memory.  With COT
// and kCotGlobal only the cotangent level and chains go to the workspace.
// Fills 1/m and m; ends with a barrier.
template <typename T, int WT, bool COT, typename Team>
__device__ __forceinline__ SigShared<T> place_arrays(const Team& tm, const SigGeometry& sg, int mode, T* gws, int64_t gws_stride,
                                                     unsigned char* smem_raw, bool& vec4, int64_t slot = -1) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t lo = G.db[D];
    const bool bwd = mode & kBackward;
    const uint32_t held = (mode & (kTopGlobal | kTopRegs)) ? lo : G.dim;  // coefficients of S kept on chip
    SigShared<T> sh;
    T* q = reinterpret_cast<T*>(smem_raw);
    // kCotGlobal: S and the forward chains in shared memory, the cotangent
    // level and chains in this CTA's slice of the global workspace
    const bool cot_global = COT && (mode & kCotGlobal) && bwd && gws;
    // the workspace slice: the CTA's, or `slot`'s (a team of the grouped launch)
    const int64_t ws_slot = slot >= 0 ? slot : static_cast<int64_t>(blockIdx.x);
    T* p = (gws && !cot_global) ? gws + ws_slot * gws_stride : q;
    // the FP32 four-coefficient forward step wants S + 1, Tf + choff[1] and the
    // scaled increments on 16-byte boundaries (kVec4; the host adds slack)
    vec4 = false;
    if constexpr (kVec4<T, WT>) vec4 = gws == nullptr && !(mode & kTopGlobal);
    const bool v4 = vec4;
    auto align4 = [&](uint32_t off) {  // elements to skip so that p + off is 16-byte aligned
        return v4 ? static_cast<uint32_t>((4u - (static_cast<uint32_t>(p - q) + off) % 4u) % 4u) : 0u;
    };
    p += align4(1);
    sh.S = p;
    sh.top = p + lo;
    p += held;
    p += align4(sg.choff[1]);
    sh.Tf = p;
    p += sg.chain_total;
    if (bwd) {
        T* g = cot_global ? gws + ws_slot * gws_stride : p;
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
    sh.lofs = 0;
    for (int m = tm.rank(); m <= D; m += tm.size()) sh.inv[m] = m == 0 ? T(0) : T(1) / static_cast<T>(m);
    for (int m = tm.rank(); m <= D + 1; m += tm.size()) sh.num[m] = static_cast<T>(m);
    tm.sync();
    return sh;
}

// One path b with increments [off, off + len): the forward pass and/or the
// reverse pass as `mode` asks.  Ends with a barrier.
// TOPREGS: the top level in registers (kTopRegs; forward-only FP32 calls).
template <typename T, int WT, bool TOPREGS = false, typename Team = CtaTeam>
__device__ __forceinline__ void run_path(const Team& tm, const SigGeometry& sg, SigShared<T>& sh, const T* __restrict__ incr,
                                         int64_t b, int64_t off, int64_t len, T* sig, int64_t sig_stride,
                                         const T* seed, int64_t seed_stride, T* grad, int mode, bool vec4) {
    const Geometry& G = sg.g;
    const int D = G.depth;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t lo = G.db[D];  // coefficients below the top level
    const bool bwd = mode & kBackward;
    const bool fwd_top = mode & kTopLevel;
    const bool top_global = mode & kTopGlobal;
    const uint32_t held = (top_global || TOPREGS) ? lo : G.dim;  // coefficients of S kept on chip
    const int nmax = fwd_top ? D : D - 1;
    const T* xin = incr + off * W;
    TopRegs<T, WT> top;
    if constexpr (TOPREGS) {
#pragma unroll
        for (int i = 0; i < kTopRows<T, WT>; ++i)
#pragma unroll
            for (int a = 0; a < WT; ++a) top[i][a] = T(0);
    }

    if (mode & kLoadFinal) {
        const T* src = sig + b * sig_stride;
        for (uint32_t i = tm.rank(); i < lo; i += tm.size()) sh.S[i] = src[i];
    } else {
        for (uint32_t i = tm.rank(); i < held; i += tm.size()) sh.S[i] = i == 0 ? T(1) : T(0);
        if (top_global && fwd_top) {
            sh.top = sig + b * sig_stride + lo;
            for (uint32_t i = tm.rank(); i < G.pw[D]; i += tm.size()) sh.top[i] = T(0);
        }
    }

    if (mode & kForward) {
        if (len > 0) set_increment(tm, sg, sh, xc_buf(sh, 0), load_increment(tm, sg, xin, 0));
        tm.sync();
        T xv = len > 1 ? load_increment(tm, sg, xin, 1) : T(0);
        for (int64_t k = 0; k < len; ++k) {
            const T x_next = xv;
            if (k + 2 < len) xv = load_increment(tm, sg, xin, k + 2);
            forward_step<T, WT, false, TOPREGS>(tm, sg, sh, xc_buf(sh, k), xc_buf(sh, k + 1), x_next, nmax,
                                                top_global, vec4, &top);
        }
        if (sig && !(mode & kLoadFinal)) {
            T* dst = sig + b * sig_stride;
            for (uint32_t i = tm.rank(); i < held; i += tm.size()) dst[i] = sh.S[i];
            if constexpr (TOPREGS) {
#pragma unroll
                for (int i = 0; i < kTopRows<T, WT>; ++i) {
                    const uint32_t r = tm.rank() + i * tm.size();
                    if (r < G.pw[D - 1])
#pragma unroll
                        for (int a = 0; a < WT; ++a) dst[lo + r * WT + a] = top[i][a];
                }
            }
        }
        tm.sync();
    }
    if (bwd) {
        const T* sd = seed + b * seed_stride;
        for (uint32_t i = tm.rank(); i < lo; i += tm.size()) sh.G[i] = sd[i];
        if (top_global)
            sh.top = const_cast<T*>(sd) + lo;  // read only in the reverse pass
        else
            for (uint32_t i = tm.rank(); i < G.pw[D]; i += tm.size()) sh.top[i] = sd[lo + i];
        T* gout = grad + off * W;
        if (len > 0) set_increment(tm, sg, sh, xc_buf(sh, len - 1), load_increment(tm, sg, xin, len - 1));
        tm.sync();
        T xv = len > 1 ? load_increment(tm, sg, xin, len - 2) : T(0);
        for (int64_t k = len - 1; k >= 0; --k) {
            const T x_next = xv;
            if (k >= 2) xv = load_increment(tm, sg, xin, k - 2);
            if (mode & kMergedReverse)
                backward_step_merged<T, WT>(tm, sg, sh, xc_buf(sh, k), xc_buf(sh, k - 1), x_next,
                                            k + 1 < len ? gout + (k + 1) * W : nullptr);
            else
                backward_step<T, WT>(tm, sg, sh, xc_buf(sh, k), xc_buf(sh, k - 1), x_next,
                                     k + 1 < len ? gout + (k + 1) * W : nullptr);
        }
        if (len > 0) {
            finish_reverse_step(tm, sg, sh, gout, false, partial_groups(tm, W));
            tm.sync();
        }
    }
    tm.sync();
}

// Log-scale key of a path's length (or cost) for the longest-first orders:
// 4 buckets per octave, so paths of similar length share a bucket.
constexpr int kLengthBuckets = 4 * 40;

__device__ __forceinline__ int length_bucket(int64_t len) {
    if (len <= 0) return 0;
    const int msb = 63 - __clzll(static_cast<unsigned long long>(len));
    const int sub = msb >= 2 ? static_cast<int>((len >> (msb - 2)) & 3) : static_cast<int>((len << (2 - msb)) & 3);
    const int key = 1 + msb * 4 + sub;
    return key < kLengthBuckets ? key : kLengthBuckets - 1;
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

}  // namespace
}  // namespace rpp_gb
