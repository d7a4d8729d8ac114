// shuffle.cu -- the shuffle algebra on batches of tensors (sm_103a).
//
// Products (include/rpp/operations/basic/st_mul.hpp, st_fma.hpp,
// st_inplace_fma.hpp, left_hs_mul.hpp; coefficient definition in
// include/rpp/operations/implementation/word_shuffle_product.hpp:43-97 and
// word_half_shuffle_product.hpp:12-56):
//   (L sh R)[w]     = sum over position subsets S of w of L[w|S] R[w|S^c]
//   (L < R)[a v]    = sum over subsets S of v of L[a (v|S)] R[v|S^c]
// Adjoints (st_adj_mul.hpp, left_hs_adj_lmul.hpp, left_hs_adj_rmul.hpp; the
// interleaving sums of operations/implementation/shuffle_adjoint_op_loop.hpp
// and word_shuffle_adjoint_multiply.hpp):
//   st_adj_mul  out[w]   = sum_u op[u] sum_{s in w sh u} arg[s]
//   hs_adj_lmul out[w]   = beta sum_a sum_u X[a u] sum_{s in w sh u} Y[a s]
//   hs_adj_rmul out[a v] = beta sum_u Y[u] sum_{s in v sh u} X[a s], out[0] = 0
// (X = integrator, Y = integrand, in the reference operator's argument order).
// tensor_pairing (tensor_pairing.hpp) is the batched dot product over the
// degrees both views hold.
//
// Every FP64 coefficient costs one FMA per (subset) term and the integer work
// that locates the two factors is kept under ~10 instructions per FMA, so the
// kernels are bound by the FP64 pipe.  Each CTA owns one tensor of the batch
// at a time (grid-stride), stages the two operands in shared memory when they
// fit and writes every output coefficient exactly once: results are
// deterministic and no atomics are used.
//
// Work order: output degrees are visited in the order the host computes
// (most expensive per coefficient first).  Degrees whose coefficients are
// expensive (the low degrees of the adjoints) give each coefficient a warp;
// the rest give each coefficient one thread, 32 consecutive coefficients per
// task.  Warps take tasks from a shared-memory counter.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>

#include "bulk_stage.cuh"
#include "launch_util.cuh"
#include "ops.hpp"

namespace rpp_gb {
namespace {

template <typename T>
__device__ __forceinline__ T warp_reduce(T v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

// Output position k of the visiting order -> (degree, index in degree).
__device__ __forceinline__ void locate(const ShuffleOrder& ord, uint32_t k, int& n, uint32_t& j) {
    int e = 0;
    while (e + 1 < ord.count && ord.start[e + 1] <= k) ++e;
    n = ord.deg[e];
    j = k - ord.start[e];
}

// ---------------------------------------------------------------------------
// Forward products.
// ---------------------------------------------------------------------------

// sum over subsets S of the m letters of v of Lget(|S|)[v|S] * R[|S^c|][v|S^c]
// where Lget(k) reads level k + e at offset a W^k (e = 1: the integrator of a
// half-shuffle with prefix letter a).  Mask bit t selects letter t counted from
// the last, as in the reference's masked packing; masks are visited in
// increasing order (high part outer, 3 low bits inner), which is the
// reference's summation order.
template <typename T, int MAXD>
__device__ T shuffle_word(const Geometry& G, int m, uint32_t v, int e, uint32_t a, const T* __restrict__ L,
                          int llo, int lhi, const T* __restrict__ R, int rlo, int rhi) {
    const uint32_t W = static_cast<uint32_t>(G.width);
    uint32_t d[MAXD];
    {
        uint32_t x = v;
#pragma unroll
        for (int t = 0; t < MAXD; ++t) {
            if (t < m) {
                uint32_t q, r;
                G.divw.divmod(x, q, r);
                d[t] = r;
                x = q;
            }
        }
    }
    const int h = m < 3 ? m : 3;
    const int nlow = 1 << h;
    // low tables: the last h letters split by each low mask
    uint32_t lowL[8], lowR[8];
#pragma unroll
    for (int lm = 0; lm < 8; ++lm) {
        uint32_t l = 0, r = 0;
#pragma unroll
        for (int t = 2; t >= 0; --t) {
            if (t < h) {
                if ((lm >> t) & 1) l = l * W + d[t];
                else r = r * W + d[t];
            }
        }
        lowL[lm] = l;
        lowR[lm] = r;
    }
    // W^c for the c low letters taken left, W^(h-c) for the h-c taken right
    uint32_t pwl[4], pwr[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        pwl[c] = G.pw[c];
        pwr[c] = c <= h ? G.pw[h - c] : 0u;
    }

    T acc = T(0);
    const uint32_t nhigh = 1u << (m - h);
    for (uint32_t hm = 0; hm < nhigh; ++hm) {
        uint32_t hl = 0, hr = 0;
        int kh = 0;
#pragma unroll
        for (int t = MAXD - 1; t >= 3; --t) {
            if (t < m) {
                if ((hm >> (t - h)) & 1u) {
                    hl = hl * W + d[t];
                    ++kh;
                } else {
                    hr = hr * W + d[t];
                }
            }
        }
        // per number c of low letters taken left: bases and validity
        uint32_t lb[4], rb[4];
        bool ok[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int kl = kh + c, kr = m - kl;
            ok[c] = c <= h && kr >= 0 && kl + e >= llo && kl + e <= lhi && kr >= rlo && kr <= rhi;
            lb[c] = ok[c] ? G.db[kl + e] + a * G.pw[kl] + hl * pwl[c] : 0u;
            rb[c] = ok[c] ? G.db[kr] + hr * pwr[c] : 0u;
        }
#pragma unroll
        for (int lm = 0; lm < 8; ++lm) {
            const int c = __builtin_popcount(lm);
            if (lm < nlow && ok[c]) acc = fma(L[lb[c] + lowL[lm]], R[rb[c] + lowR[lm]], acc);
        }
    }
    return acc;
}

// Scale: beta != 1, multiplied in per coefficient (a compile-time choice:
// as a run-time select the multiply ran for every coefficient).
template <typename T, int MAXD, bool Scale>
__global__ void __launch_bounds__(256) k_shuffle_product(Geometry G, int kind, TArg<T> out, TArg<T> add, TArg<T> lhs,
                                                        TArg<T> rhs, int64_t batch, T alpha, T beta, int staged,
                                                        ShuffleOrder ord) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* sm = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    const uint32_t pd = staged_elems<T>(G.dim);
    uint32_t phase = 0;
    if (staged) bulk_stage_init(bar);
    __shared__ uint32_t s_next;
    const int e = kind == static_cast<int>(ShuffleKind::LeftHalf) ? 1 : 0;
    const int lhi = imin(lhs.hi, G.depth), rhi = imin(rhs.hi, G.depth);
    const uint32_t total = ord.start[ord.count];
    const uint32_t ntasks = (total + 31) / 32;
    const int lane = threadIdx.x & 31;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const T* L = lhs.at(b);
        const T* R = rhs.at(b);
        T* o = out.at(b);
        const T* A = add.p ? add.at(b) : nullptr;
        if (threadIdx.x == 0) s_next = 0;
        if (staged) {
            BulkStage<T> st(bar, phase);
            L = st.add(sm, L, lhs.lo, lhi, G);
            R = st.add(sm + pd, R, rhs.lo, rhi, G);
            if (!st.commit(G.fault)) return;
        } else {
            __syncthreads();
        }
        for (;;) {
            uint32_t t = 0;
            if (lane == 0) t = atomicAdd(&s_next, 1u);
            t = __shfl_sync(0xffffffffu, t, 0);
            if (t >= ntasks) break;
            const uint32_t k = t * 32 + lane;
            if (k < total) {
                int n;
                uint32_t j;
                locate(ord, k, n, j);
                T val;
                if (e) {
                    if (n == 0) {
                        val = T(0);
                    } else {
                        const uint32_t tail = G.pw[n - 1];
                        const uint32_t a = j / tail, v = j - a * tail;
                        val = shuffle_word<T, MAXD>(G, n - 1, v, 1, a, L, lhs.lo, lhi, R, rhs.lo, rhi);
                        if constexpr (Scale) val *= beta;
                    }
                } else {
                    val = shuffle_word<T, MAXD>(G, n, j, 0, 0u, L, lhs.lo, lhi, R, rhs.lo, rhi);
                    if constexpr (Scale) val *= beta;
                    if (kind == static_cast<int>(ShuffleKind::InplaceFma)) {
                        val = fma(alpha, o[G.db[n] + j], val);
                    } else if (kind == static_cast<int>(ShuffleKind::Fma) && A && add.has(n)) {
                        val = fma(alpha, A[G.db[n] + j], val);
                    }
                }
                o[G.db[n] + j] = val;
            }
        }
        bulk_stage_reuse();
    }
}

// ---------------------------------------------------------------------------
// Adjoints.
// ---------------------------------------------------------------------------

// The terms of one adjoint coefficient are grouped in items (m, a, M, u_hi):
// prefix letter a (the left adjoint's letter loop; a single fixed letter or
// none otherwise), op degree m, interleaving mask M of weight m on the
// nw + m positions of the merged word (bit b = position b counted from the
// last letter) and the high part u_hi of the op word u = u_hi W^k + u_lo,
// k = min(m, 2).  An item sums over the k last letters u_lo:
//     OP[ob(a, m) + u] * ARG[ab(a, m) + merge(w, u, M)]
// (W^k terms; one when m = 0), so the walk that places w's and u_hi's
// letters is paid once per W^k FMAs.  Items are visited op degree first,
// highest degree (largest items) first, then mask, u_hi and letter, so that
// lanes taking every 32nd item get the large items first and balance.  A
// cursor walks the items in that order; lanes of a warp take every 32nd item,
// a single thread takes them all.  Skipping ahead costs one Gosper step per
// mask passed; with the letter innermost, a lane of the left adjoint passes
// 32/W (mask, u_hi) pairs per item instead of 32 (letter outside the mask,
// every mask of a low degree one pair).
struct AdjItems {
    int kind;
    int nw;       // letters of the output word w (after the rmul prefix)
    uint32_t w;   // its index within its degree
    int a0, a1;   // letter range [a0, a1)
    int mlo, mhi; // op degree range
    // cursor
    int a, m;
    uint32_t M, last, nhi, uh;
    bool done;

    __device__ void start_degree(const Geometry& G) {
        M = (1u << m) - 1u;
        last = M << nw;
        nhi = m <= 1 ? 1u : G.pw[m - 2];
    }
    __device__ bool next_mask(const Geometry& G) {
        if (M != last) {
            const uint32_t low = M & (0u - M);
            const uint32_t ripple = M + low;
            M = ripple | (((ripple ^ M) >> 2) >> (__ffs(M) - 1));
            return true;
        }
        if (--m < mlo) return false;
        start_degree(G);
        return true;
    }
    __device__ void init(const Geometry& G, uint32_t first) {
        a = a0;
        m = mhi;
        uh = 0;
        done = mlo > mhi || a0 >= a1;
        if (!done) {
            start_degree(G);
            advance(G, first);
        }
    }
    __device__ void advance(const Geometry& G, uint32_t k) {
        // k items on: the letter is the innermost digit (a1 - a0 = 1 or W)
        uint32_t carry = k;
        if (a1 - a0 > 1) {
            uint32_t r;
            G.divw.divmod(static_cast<uint32_t>(a - a0) + k, carry, r);
            a = a0 + static_cast<int>(r);
        }
        uh += carry;
        while (uh >= nhi) {
            uh -= nhi;
            if (!next_mask(G)) {
                done = true;
                return;
            }
        }
    }
};

// The W^k FMAs of one item for letter a (k = min(m, 2); m >= 1): op words
// uh*W^2 + u1*W + u0 (m >= 2) or u0 (m = 1), argument at `ar` + u0*c0 + u1*c1.
template <typename T>
__device__ __forceinline__ T item_terms(const T* __restrict__ op, const T* __restrict__ ar, uint32_t W, int m,
                                        uint32_t c0, uint32_t c1, T acc) {
    if (m >= 2) {
        for (uint32_t u1 = 0; u1 < W; ++u1, op += W, ar += c1)
            for (uint32_t u0 = 0; u0 < W; ++u0) acc = fma(op[u0], ar[u0 * c0], acc);
    } else {
        for (uint32_t u0 = 0; u0 < W; ++u0) acc = fma(op[u0], ar[u0 * c0], acc);
    }
    return acc;
}

template <typename T>
__device__ T adjoint_coeff(const Geometry& G, int kind, int n, uint32_t j, const T* __restrict__ OP, int olo,
                           int ohi, const T* __restrict__ ARG, int alo, int ahi, uint32_t first, uint32_t step) {
    const uint32_t W = static_cast<uint32_t>(G.width);
    AdjItems it;
    it.kind = kind;
    if (kind == static_cast<int>(ShuffleAdjKind::HalfL)) {
        it.nw = n;
        it.w = j;
        it.a0 = 0;
        it.a1 = static_cast<int>(W);
        it.mlo = imax(0, imax(olo - 1, alo - 1 - n));
        it.mhi = imin(ohi - 1, ahi - 1 - n);
    } else if (kind == static_cast<int>(ShuffleAdjKind::HalfR)) {
        if (n == 0) return T(0);
        const uint32_t tail = G.pw[n - 1];
        const uint32_t a = j / tail;
        it.nw = n - 1;
        it.w = j - a * tail;
        it.a0 = static_cast<int>(a);
        it.a1 = it.a0 + 1;
        it.mlo = imax(olo, alo - n);
        it.mhi = imin(ohi, ahi - n);
    } else {
        it.nw = n;
        it.w = j;
        it.a0 = 0;
        it.a1 = 1;
        it.mlo = imax(olo, alo - n);
        it.mhi = imin(ohi, ahi - n);
    }
    it.init(G, first);
    T acc = T(0);
    while (!it.done) {
        const int m = it.m, N = it.nw + m;
        const uint32_t a = static_cast<uint32_t>(it.a);
        uint32_t ob, ab;
        if (kind == static_cast<int>(ShuffleAdjKind::HalfL)) {
            ob = G.db[m + 1] + a * G.pw[m];
            ab = G.db[N + 1] + a * G.pw[N];
        } else if (kind == static_cast<int>(ShuffleAdjKind::HalfR)) {
            ob = G.db[m];
            ab = G.db[N + 1] + a * G.pw[N];
        } else {
            ob = G.db[m];
            ab = G.db[N];
        }
        if (m == 0) {
            acc = fma(OP[ob], ARG[ab + it.w], acc);
        } else {
            // the k lowest set bits of M carry u_lo; the rest of M carries u_hi
            const uint32_t M = it.M;
            const uint32_t b0 = M & (0u - M);
            const uint32_t r0 = M ^ b0;
            const uint32_t b1 = m >= 2 ? r0 & (0u - r0) : 0u;
            const uint32_t rest = r0 ^ b1;
            const uint32_t c0 = G.pw[__ffs(b0) - 1];
            uint32_t wq = it.w, uq = it.uh, base = 0, p = 1;
            for (int bpos = 0; bpos < N; ++bpos) {
                const uint32_t bit = 1u << bpos;
                if (!((b0 | b1) & bit)) {
                    const bool from_u = (rest & bit) != 0;
                    const uint32_t src = from_u ? uq : wq;
                    uint32_t q, r;
                    G.divw.divmod(src, q, r);
                    if (from_u) uq = q;
                    else wq = q;
                    base += r * p;
                }
                p *= W;
            }
            if (m >= 2) {
                const uint32_t c1 = G.pw[__ffs(b1) - 1];
                const T* op = OP + ob + it.uh * W * W;
                const T* ar = ARG + ab + base;
                for (uint32_t u1 = 0; u1 < W; ++u1, op += W, ar += c1)
                    for (uint32_t u0 = 0; u0 < W; ++u0) acc = fma(op[u0], ar[u0 * c0], acc);
            } else {
                const T* op = OP + ob;
                const T* ar = ARG + ab + base;
                for (uint32_t u0 = 0; u0 < W; ++u0) acc = fma(op[u0], ar[u0 * c0], acc);
            }
        }
        it.advance(G, step);
    }
    return acc;
}

// The same sum for one thread alone: plain nested loops over (a, m, M, u_hi),
// the cursor's order, without its per-item bookkeeping (most coefficients of
// high degree hold single-term items).
template <typename T>
__device__ T adjoint_coeff_seq(const Geometry& G, int kind, int n, uint32_t j, const T* __restrict__ OP, int olo,
                               int ohi, const T* __restrict__ ARG, int alo, int ahi) {
    const uint32_t W = static_cast<uint32_t>(G.width);
    int nw = n, a0 = 0, a1 = 1, mlo, mhi;
    uint32_t w = j;
    if (kind == static_cast<int>(ShuffleAdjKind::HalfL)) {
        a1 = static_cast<int>(W);
        mlo = imax(0, imax(olo - 1, alo - 1 - n));
        mhi = imin(ohi - 1, ahi - 1 - n);
    } else if (kind == static_cast<int>(ShuffleAdjKind::HalfR)) {
        if (n == 0) return T(0);
        const uint32_t tail = G.pw[n - 1];
        const uint32_t a = j / tail;
        nw = n - 1;
        w = j - a * tail;
        a0 = static_cast<int>(a);
        a1 = a0 + 1;
        mlo = imax(olo, alo - n);
        mhi = imin(ohi, ahi - n);
    } else {
        mlo = imax(olo, alo - n);
        mhi = imin(ohi, ahi - n);
    }
    T acc = T(0);
    for (int ai = a0; ai < a1; ++ai) {
        const uint32_t a = static_cast<uint32_t>(ai);
        for (int m = mlo; m <= mhi; ++m) {
            const int N = nw + m;
            uint32_t ob, ab;
            if (kind == static_cast<int>(ShuffleAdjKind::HalfL)) {
                ob = G.db[m + 1] + a * G.pw[m];
                ab = G.db[N + 1] + a * G.pw[N];
            } else if (kind == static_cast<int>(ShuffleAdjKind::HalfR)) {
                ob = G.db[m];
                ab = G.db[N + 1] + a * G.pw[N];
            } else {
                ob = G.db[m];
                ab = G.db[N];
            }
            if (m == 0) {
                acc = fma(OP[ob], ARG[ab + w], acc);
                continue;
            }
            const uint32_t nhi = m <= 1 ? 1u : G.pw[m - 2];
            uint32_t M = (1u << m) - 1u;
            const uint32_t last = M << nw;
            for (;;) {
                const uint32_t b0 = M & (0u - M);
                const uint32_t r0 = M ^ b0;
                const uint32_t b1 = m >= 2 ? r0 & (0u - r0) : 0u;
                const uint32_t rest = r0 ^ b1;
                const uint32_t c0 = G.pw[__ffs(b0) - 1];
                const uint32_t c1 = m >= 2 ? G.pw[__ffs(b1) - 1] : 0u;
                for (uint32_t uh = 0; uh < nhi; ++uh) {
                    uint32_t wq = w, uq = uh, base = 0, p = 1;
                    for (int bpos = 0; bpos < N; ++bpos) {
                        const uint32_t bit = 1u << bpos;
                        if (!((b0 | b1) & bit)) {
                            const bool from_u = (rest & bit) != 0;
                            const uint32_t src = from_u ? uq : wq;
                            uint32_t q, r;
                            G.divw.divmod(src, q, r);
                            if (from_u) uq = q;
                            else wq = q;
                            base += r * p;
                        }
                        p *= W;
                    }
                    const T* ar = ARG + ab + base;
                    if (m >= 2) {
                        const T* op = OP + ob + uh * W * W;
                        for (uint32_t u1 = 0; u1 < W; ++u1, op += W, ar += c1)
                            for (uint32_t u0 = 0; u0 < W; ++u0) acc = fma(op[u0], ar[u0 * c0], acc);
                    } else {
                        const T* op = OP + ob;
                        for (uint32_t u0 = 0; u0 < W; ++u0) acc = fma(op[u0], ar[u0 * c0], acc);
                    }
                }
                if (M == last) break;
                const uint32_t ripple = M + b0;
                M = ripple | (((ripple ^ M) >> 2) >> (__ffs(M) - 1));
            }
        }
    }
    return acc;
}

// The left adjoint's sum for one thread alone: plain nested loops over
// (m, M, u_hi), with the prefix letters innermost -- the walk that places w's
// and u_hi's letters is the same for every letter a, so a thread pays it once
// per W x W^k FMAs.  (The warp cursor keeps the letter in the item key: items
// W times larger would leave the lanes of a low-degree coefficient's warp
// unbalanced -- measured 39 % slower on left_hs_adj_lmul at W5 D5.)  Letter
// a's op block of degree m + 1 starts at db[m+1] + a W^m, its argument block
// of degree n + m + 1 at db[n+m+1] + a W^{n+m}.
template <typename T>
__device__ T adjoint_coeff_seq_left(const Geometry& G, int n, uint32_t w, const T* __restrict__ OP, int olo,
                                    int ohi, const T* __restrict__ ARG, int alo, int ahi) {
    const uint32_t W = static_cast<uint32_t>(G.width);
    const int mlo = imax(0, imax(olo - 1, alo - 1 - n));
    const int mhi = imin(ohi - 1, ahi - 1 - n);
    T acc = T(0);
    for (int m = mhi; m >= mlo; --m) {
        const int N = n + m;
        const uint32_t ob0 = G.db[m + 1], obs = G.pw[m], ab0 = G.db[N + 1], abs = G.pw[N];
        if (m == 0) {
            for (uint32_t a = 0; a < W; ++a) acc = fma(OP[ob0 + a * obs], ARG[ab0 + a * abs + w], acc);
            continue;
        }
        const uint32_t nhi = m <= 1 ? 1u : G.pw[m - 2];
        uint32_t M = (1u << m) - 1u;
        const uint32_t last = M << n;
        for (;;) {
            const uint32_t b0 = M & (0u - M);
            const uint32_t r0 = M ^ b0;
            const uint32_t b1 = m >= 2 ? r0 & (0u - r0) : 0u;
            const uint32_t rest = r0 ^ b1;
            const uint32_t c0 = G.pw[__ffs(b0) - 1];
            const uint32_t c1 = m >= 2 ? G.pw[__ffs(b1) - 1] : 0u;
            for (uint32_t uh = 0; uh < nhi; ++uh) {
                uint32_t wq = w, uq = uh, base = 0, p = 1;
                for (int bpos = 0; bpos < N; ++bpos) {
                    const uint32_t bit = 1u << bpos;
                    if (!((b0 | b1) & bit)) {
                        const bool from_u = (rest & bit) != 0;
                        const uint32_t src = from_u ? uq : wq;
                        uint32_t q, r;
                        G.divw.divmod(src, q, r);
                        if (from_u) uq = q;
                        else wq = q;
                        base += r * p;
                    }
                    p *= W;
                }
                const uint32_t ou = m >= 2 ? uh * W * W : 0u;
                for (uint32_t a = 0; a < W; ++a)
                    acc = item_terms(OP + ob0 + a * obs + ou, ARG + ab0 + a * abs + base, W, m, c0, c1, acc);
            }
            if (M == last) break;
            const uint32_t ripple = M + b0;
            M = ripple | (((ripple ^ M) >> 2) >> (__ffs(M) - 1));
        }
    }
    return acc;
}

// Scale: beta != 1 (compile time; as a run-time select the FP64 multiply ran
// for every output coefficient: 7 % of the DFMA count of left_hs_adj_lmul at
// W5 D5).
template <typename T, bool Scale>
__global__ void __launch_bounds__(256, 3) k_shuffle_adjoint(Geometry G, int kind, TArg<T> out, TArg<T> op,
                                                        TArg<T> arg, int64_t batch, T beta, int staged,
                                                        ShuffleOrder ord) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* sm = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    const uint32_t pd = staged_elems<T>(G.dim);
    uint32_t phase = 0;
    if (staged) bulk_stage_init(bar);
    __shared__ uint32_t s_next;
    const int ohi = imin(op.hi, G.depth), ahi = imin(arg.hi, G.depth);
    const uint32_t nwarp = ord.start[ord.warp_entries];
    const uint32_t total = ord.start[ord.tasked];
    const uint32_t ntasks = nwarp + (total - nwarp + 31) / 32;
    const int lane = threadIdx.x & 31;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const T* P = op.at(b);
        const T* A = arg.at(b);
        T* o = out.at(b);
        if (threadIdx.x == 0) s_next = 0;
        if (staged) {
            BulkStage<T> st(bar, phase);
            P = st.add(sm, P, op.lo, ohi, G);
            A = st.add(sm + pd, A, arg.lo, ahi, G);
            if (!st.commit(G.fault)) return;
        } else {
            __syncthreads();
        }
        // degrees without terms (e.g. the top degree of the left adjoint):
        // coalesced zero stores by the whole CTA instead of one queued task
        // per 32 coefficients (after the inputs are read or staged, as every
        // other write)
        for (int i = ord.tasked; i < ord.count; ++i) {
            T* z = o + G.db[ord.deg[i]];
            const uint32_t len = G.pw[ord.deg[i]];
            for (uint32_t u = threadIdx.x; u < len; u += blockDim.x) z[u] = T(0);
        }
        for (;;) {
            uint32_t t = 0;
            if (lane == 0) t = atomicAdd(&s_next, 1u);
            t = __shfl_sync(0xffffffffu, t, 0);
            if (t >= ntasks) break;
            if (t < nwarp) {
                int n;
                uint32_t j;
                locate(ord, t, n, j);
                T acc = adjoint_coeff<T>(G, kind, n, j, P, op.lo, ohi, A, arg.lo, ahi, lane, 32);
                acc = warp_reduce(acc);
                if (lane == 0) o[G.db[n] + j] = Scale ? beta * acc : acc;
            } else {
                const uint32_t k = nwarp + (t - nwarp) * 32 + lane;
                if (k < total) {
                    int n;
                    uint32_t j;
                    locate(ord, k, n, j);
                    const T acc = kind == static_cast<int>(ShuffleAdjKind::HalfL)
                                      ? adjoint_coeff_seq_left<T>(G, n, j, P, op.lo, ohi, A, arg.lo, ahi)
                                      : adjoint_coeff_seq<T>(G, kind, n, j, P, op.lo, ohi, A, arg.lo, ahi);
                    o[G.db[n] + j] = Scale ? beta * acc : acc;
                }
            }
        }
        bulk_stage_reuse();
    }
}

// tensor_pairing: one warp per tensor of the batch (HBM-bound).
template <typename T>
__global__ void k_pairing(const T* __restrict__ F, int64_t fs, const T* __restrict__ A, int64_t as, T* result,
                          uint32_t begin, uint32_t end, int64_t batch) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
    for (int64_t b = blockIdx.x * static_cast<int64_t>(blockDim.x >> 5) + (threadIdx.x >> 5); b < batch;
         b += warps) {
        const T* f = F + b * fs;
        const T* a = A + b * as;
        T acc = T(0);
        for (uint32_t i = begin + lane; i < end; i += 32) acc = fma(f[i], a[i], acc);
        acc = warp_reduce(acc);
        if (lane == 0) result[b] = acc;
    }
}

constexpr size_t kStageLimit = 200 * 1024;

template <typename Kernel>
cudaError_t shuffle_launch_shape(Kernel kernel, const Geometry& g, const DeviceInfo& dev, size_t elem, int64_t batch,
                                 int& threads, size_t& smem, int& staged, dim3& grid) {
    const size_t per16 = 16 / elem;  // staged buffers: padded for the bulk copy's alignment shift
    const size_t need = kBulkHeader + 2 * ((g.dim + 2 * per16 - 1) / per16 * per16) * elem;
    staged = need <= kStageLimit && need <= static_cast<size_t>(dev.max_smem_optin) ? 1 : 0;
    smem = staged ? need : 0;
    threads = threads_for(g.pw[g.depth]);
    if (threads < 64) threads = 64;
    return batch_grid(kernel, dev, threads, smem, batch, grid);
}

}  // namespace

ShuffleOrder shuffle_product_order(const Geometry& g, int out_lo, int out_hi) {
    // a coefficient of degree n costs 2^n terms: visit the top degree first
    ShuffleOrder o{};
    const int hi = out_hi < g.depth ? out_hi : g.depth;
    uint32_t acc = 0;
    for (int n = hi; n >= out_lo && n >= 0; --n) {
        o.deg[o.count] = n;
        o.start[o.count] = acc;
        acc += g.pw[n];
        ++o.count;
    }
    o.start[o.count] = acc;
    o.tasked = o.count;
    return o;
}

ShuffleOrder shuffle_adjoint_order(const Geometry& g, ShuffleAdjKind kind, int out_lo, int out_hi, int op_lo,
                                   int op_hi, int arg_lo, int arg_hi, int threads) {
    // Terms per coefficient of degree n: sum over op degrees m of
    // C(nw + m, m) W^m (times W for the left adjoint's letter loop).  A
    // coefficient gets a warp when one thread alone would take more than
    // twice the CTA's mean work per thread (and at least 128 terms).
    struct Entry {
        int n;
        double cost;
    };
    Entry e[kMaxDepth + 1];
    int count = 0;
    const int D = g.depth;
    const int ohi = op_hi < D ? op_hi : D, ahi = arg_hi < D ? arg_hi : D;
    const double W = static_cast<double>(g.width);
    for (int n = out_lo < 0 ? 0 : out_lo; n <= out_hi && n <= D; ++n) {
        int lo, hi, nw = n;
        if (kind == ShuffleAdjKind::HalfL) {
            lo = std::max({0, op_lo - 1, arg_lo - 1 - n});
            hi = std::min(ohi - 1, ahi - 1 - n);
        } else {
            lo = std::max(op_lo, arg_lo - n);
            hi = std::min(ohi, ahi - n);
            if (kind == ShuffleAdjKind::HalfR) nw = n - 1;
        }
        double cost = 0.0;
        if (!(kind == ShuffleAdjKind::HalfR && n == 0)) {
            for (int m = lo < 0 ? 0 : lo; m <= hi; ++m) {
                double c = 1.0;  // C(nw + m, m)
                for (int i = 1; i <= m; ++i) c = c * (nw + i) / i;
                cost += c * std::pow(W, m);
            }
            if (kind == ShuffleAdjKind::HalfL) cost *= W;
        }
        e[count++] = {n, cost};
    }
    double total = 0.0;
    for (int i = 0; i < count; ++i) total += e[i].cost * g.pw[e[i].n];
    const double kWarpTerms = std::max(128.0, 2.0 * total / std::max(1, threads));
    std::stable_sort(e, e + count, [](const Entry& x, const Entry& y) { return x.cost > y.cost; });
    ShuffleOrder o{};
    uint32_t acc = 0;
    for (int i = 0; i < count; ++i) {
        o.deg[i] = e[i].n;
        o.start[i] = acc;
        acc += g.pw[e[i].n];
        if (e[i].cost >= kWarpTerms && o.warp_entries == i) o.warp_entries = i + 1;
    }
    o.count = count;
    o.start[count] = acc;
    o.tasked = count;
    while (o.tasked > o.warp_entries && e[o.tasked - 1].cost == 0.0) --o.tasked;
    return o;
}

template <typename T>
cudaError_t launch_shuffle_product(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, ShuffleKind kind,
                                   TArg<T> out, TArg<T> add, TArg<T> lhs, TArg<T> rhs, int64_t batch, double alpha,
                                   double beta, const ShuffleOrder& ord) {
    if (batch <= 0 || ord.start[ord.count] == 0) return cudaSuccess;
    if (g.depth > 30) return cudaErrorInvalidValue;
    int threads, staged;
    size_t smem;
    dim3 grid;
    cudaError_t err;
#define RPP_GB_SHUFFLE_FWD(MAXD, SCALE)                                                                    \
    {                                                                                                      \
        constexpr auto kernel = k_shuffle_product<T, MAXD, SCALE>;                                         \
        if ((err = allow_large_smem<kernel>(dev)) != cudaSuccess) return err;                              \
        if ((err = shuffle_launch_shape(kernel, g, dev, sizeof(T), batch, threads, smem, staged, grid)) != \
            cudaSuccess)                                                                                   \
            return err;                                                                                    \
        kernel<<<grid, threads, smem, s>>>(g, static_cast<int>(kind), out, add, lhs, rhs, batch,           \
                                           static_cast<T>(alpha), static_cast<T>(beta), staged, ord);      \
    }
    const bool scale = static_cast<T>(beta) != T(1);
    if (g.depth <= 8) {
        if (scale) RPP_GB_SHUFFLE_FWD(8, true) else RPP_GB_SHUFFLE_FWD(8, false)
    } else if (g.depth <= 16) {
        if (scale) RPP_GB_SHUFFLE_FWD(16, true) else RPP_GB_SHUFFLE_FWD(16, false)
    } else {
        if (scale) RPP_GB_SHUFFLE_FWD(32, true) else RPP_GB_SHUFFLE_FWD(32, false)
    }
#undef RPP_GB_SHUFFLE_FWD
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_shuffle_adjoint(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, ShuffleAdjKind kind,
                                   TArg<T> out, TArg<T> op, TArg<T> arg, int64_t batch, double beta) {
    if (batch <= 0) return cudaSuccess;
    auto run = [&](auto kernel_c) -> cudaError_t {
        constexpr auto kernel = decltype(kernel_c)::value;
        cudaError_t err = allow_large_smem<kernel>(dev);
        if (err != cudaSuccess) return err;
        int threads, staged;
        size_t smem;
        dim3 grid;
        if ((err = shuffle_launch_shape(kernel, g, dev, sizeof(T), batch, threads, smem, staged, grid)) !=
            cudaSuccess)
            return err;
        const ShuffleOrder ord =
            shuffle_adjoint_order(g, kind, out.lo, out.hi, op.lo, op.hi, arg.lo, arg.hi, threads);
        if (ord.start[ord.count] == 0) return cudaSuccess;
        kernel<<<grid, threads, smem, s>>>(g, static_cast<int>(kind), out, op, arg, batch, static_cast<T>(beta),
                                           staged, ord);
        return cudaGetLastError();
    };
    if (static_cast<T>(beta) == T(1))
        return run(std::integral_constant<decltype(&k_shuffle_adjoint<T, false>), &k_shuffle_adjoint<T, false>>{});
    return run(std::integral_constant<decltype(&k_shuffle_adjoint<T, true>), &k_shuffle_adjoint<T, true>>{});
}

template <typename T>
cudaError_t launch_pairing(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, T* result, TArg<T> f, TArg<T> a,
                           int64_t batch) {
    if (batch <= 0) return cudaSuccess;
    const int lo = f.lo > a.lo ? f.lo : a.lo;
    int hi = f.hi < a.hi ? f.hi : a.hi;
    if (hi > g.depth) hi = g.depth;
    const uint32_t begin = lo <= hi ? g.db[lo] : 0u, end = lo <= hi ? g.db[hi + 1] : 0u;
    const int threads = 256;
    const int64_t blocks_needed = (batch + 7) / 8;
    const int64_t cap = static_cast<int64_t>(dev.sm_count) * 8;
    const unsigned blocks = static_cast<unsigned>(blocks_needed < cap ? blocks_needed : cap);
    k_pairing<T><<<blocks, threads, 0, s>>>(f.p, f.stride, a.p, a.stride, result, begin, end, batch);
    return cudaGetLastError();
}

#define RPP_GB_INSTANTIATE_SHUFFLE(T)                                                                           \
    template cudaError_t launch_shuffle_product<T>(const Geometry&, const DeviceInfo&, cudaStream_t, ShuffleKind, \
                                                   TArg<T>, TArg<T>, TArg<T>, TArg<T>, int64_t, double, double,   \
                                                   const ShuffleOrder&);                                          \
    template cudaError_t launch_shuffle_adjoint<T>(const Geometry&, const DeviceInfo&, cudaStream_t,              \
                                                   ShuffleAdjKind, TArg<T>, TArg<T>, TArg<T>, int64_t, double);   \
    template cudaError_t launch_pairing<T>(const Geometry&, const DeviceInfo&, cudaStream_t, T*, TArg<T>, TArg<T>, \
                                           int64_t);

RPP_GB_INSTANTIATE_SHUFFLE(float)
RPP_GB_INSTANTIATE_SHUFFLE(double)

}  // namespace rpp_gb
