// signature_letters.cuh -- the FP32 forward step with one warp per first
// letter (k_signature_letters in signature_fp32.cu, and FP32 forward-only
// jobs of the grouped launch in signature_group.cu).
//
// The same Chen step as signature_body.cuh (Horner chains
// T^n_j = S_j + T^n_{j-1} (x) x / (n-j+1), S_n <- T^n_n), organised for FP32,
// where the shared-memory kernel is bound by instruction issue (about twelve
// instructions per FFMA at W8 D4: the loop and index bookkeeping of the small
// lower levels and a CTA barrier per stage).  Here:
//  * A CTA of W warps runs one path; warp c holds the coefficients whose
//    first letter is c (W^{j-1} of level j).  A coefficient's Horner parent is
//    its prefix, which has the same first letter, so the warps never exchange
//    data during the path (the slicing of the cluster-split kernel, at warp
//    granularity).
//  * Each lane evaluates the Horner chains of its own coefficients from the
//    old lower levels (letter_step): no chain arrays and no stage barriers,
//    two __syncwarp per step.
//  * Width and depth are compile-time, so every stage, chain offset, level
//    size and index split is a constant and the loops unroll.
//  * The top level lives in registers: lane l holds the rows l, l + 32, ... of
//    the warp's slice (W coefficients sharing one prefix), so one chain value
//    serves W FMAs with the increment in registers.  No chain reads the top
//    level, so no other thread needs it.  Level D-1 lives in registers too:
//    lane l holds its coefficients l, l + 32, ..., which are exactly the
//    prefixes of its top rows and are read by no other lane.
//  * The increment's W letters are double-buffered by step parity in shared
//    memory; x_a / m is formed in a register as x_a * (1/m), the single
//    rounding the shared-memory kernel's scaled increments get.  Each lane
//    a < W loads its letter eight steps ahead into a register ring (a step
//    here is short, and a load one step ahead left the L2 latency exposed).
// The arithmetic is the shared-memory kernel's (the same chains and scale
// factors), summed in the same order per coefficient.
#pragma once

#include "signature_body.cuh"

namespace rpp_gb {
namespace {


// W^n as a loop, not a recursion: inlined into the unrolled stage loops it
// folds to a constant, so the index splits below are multiply-shifts (a
// recursive form was not inlined, leaving run-time divisions in every step).
constexpr uint32_t cpow(uint32_t w, int n) {
    uint32_t r = 1;
    for (int i = 0; i < n; ++i) r *= w;
    return r;
}

// Per-warp layout (floats): two buffers of scaled increments (each padded to
// a multiple of four floats, so the top's W letters load as float4), then the
// slices of the levels kept in shared memory, 1..D-2 (level D-1 lives in
// registers; at D = 2 level 1 stays in shared memory).  Each warp's region is a
// multiple of four floats, so every buffer starts on a 16-byte boundary.
template <int W, int D>
struct LetterLayout {
    static constexpr uint32_t slice(int j) { return cpow(W, j - 1); }  // level j >= 1
    static constexpr uint32_t s_off(int j) {                            // level j in S, 1 <= j
        uint32_t o = 0;
        for (int i = 1; i < j; ++i) o += slice(i);
        return o;
    }
    static constexpr bool reg_dm1 = D >= 3;                // level D-1 in registers
    static constexpr int smem_levels = reg_dm1 ? D - 2 : D - 1;
    static constexpr uint32_t s_size = s_off(smem_levels + 1);
    static constexpr uint32_t xcs = (W + 3) / 4 * 4;       // one increment buffer (x_a)
    static constexpr uint32_t warp_floats = (2 * xcs + s_size + 3) / 4 * 4;
    static constexpr uint32_t top_rows = slice(D - 1);                      // rows of W on top
    static constexpr int rows_per_lane = static_cast<int>((top_rows + 31) / 32);
};

// Full tensor level start db[j] = (W^j - 1) / (W - 1) (W >= 2).
template <int W>
constexpr uint32_t level_start(int j) {
    uint32_t s = 0;
    for (int i = 0; i < j; ++i) s += cpow(W, i);
    return s;
}

// Lower-level coefficients (levels 1..D-1 of the warp's slice) a lane
// updates per step: ceil(W^{n-1} / 32) of level n.
template <int W, int D>
constexpr int lower_per_lane() {
    int t = 0;
    for (int n = 1; n <= LetterLayout<W, D>::smem_levels; ++n) t += static_cast<int>((cpow(W, n - 1) + 31) / 32);
    return t;
}

// One forward step of warp c (its first-letter slice).  Every coefficient's
// Horner chain is evaluated by the lane that updates it, from the old lower
// levels: for a word (c, a_2, ..., a_n) of level n,
//     T_1 = S_1 + x_c / n,   T_j = S_j[a_1..a_j] + T_{j-1} x_{a_j} / (n-j+1),
// and the new S_n is T_n (the top level adds T_{D-1} x_a to its registers).
// These are the shared-memory kernel's chain values, formed by the same fused
// multiply-adds in the same order, so the results are identical; only the
// sharing of a prefix's chain value between coefficients is given up (17 %
// more FMAs at W8 D4), for no chain arrays, no stage barriers and little
// index arithmetic.  All lanes read the old levels before any lane writes the
// new ones (one __syncwarp between); the caller's __syncwarp after refreshing
// the increment orders the writes before the next step's reads.
template <int W, int D>
__device__ __forceinline__ void letter_step(float* S, const float* x,
                                            float (&top)[LetterLayout<W, D>::rows_per_lane][W],
                                            float (&sd)[LetterLayout<W, D>::rows_per_lane], uint32_t c,
                                            uint32_t lane) {
    using Lay = LetterLayout<W, D>;
    constexpr int R = Lay::rows_per_lane;
    constexpr int NS = Lay::smem_levels;  // levels in shared memory: 1..NS
    // x_a / m is formed in a register as x_a * (1/m) with __fmul_rn: the one
    // rounding the shared-memory kernel's scaled increments get (1/m is the
    // correctly rounded constant, as that kernel's 1/m table is), and no
    // contraction of the product into a following add
    const float s1 = NS >= 1 ? S[Lay::s_off(1)] : 0.0f;
    const float xcc = x[c];
    float t1[D + 1];  // T^n_1 = S_1 + S_0 x_c / n (S_0 = 1)
#pragma unroll
    for (int n = 2; n <= D; ++n) t1[n] = s1 + __fmul_rn(xcc, 1.0f / static_cast<float>(n));
    float nv[lower_per_lane<W, D>() > 0 ? lower_per_lane<W, D>() : 1];
    int v = 0;
    // level 1: S_1 + S_0 x_c
    nv[v++] = s1 + xcc;
    // levels 2..NS in shared memory
#pragma unroll
    for (int n = 2; n <= NS; ++n) {
        const uint32_t sl = Lay::slice(n);
#pragma unroll
        for (uint32_t q = 0; q < (sl + 31) / 32; ++q, ++v) {
            const uint32_t u = lane + 32u * q;
            if (u < sl) {
                float acc = t1[n];
#pragma unroll
                for (int j = 2; j <= n; ++j) {
                    const uint32_t pref = u / cpow(W, n - j);  // index of (c, a_2..a_j) in level j's slice
                    const float xm = __fmul_rn(x[pref % W], 1.0f / static_cast<float>(n - j + 1));
                    acc = fmaf(acc, xm, S[Lay::s_off(j) + pref]);
                }
                nv[v] = acc;
            }
        }
    }
    // level D-1 in registers (lane owns coefficients lane + 32 r, which are
    // also the prefixes of its top rows) and the top rows
    float x1[W];
    if constexpr (W % 4 == 0) {
#pragma unroll
        for (int a = 0; a < W; a += 4) {
            const float4 x4 = *reinterpret_cast<const float4*>(x + a);
            x1[a] = x4.x;
            x1[a + 1] = x4.y;
            x1[a + 2] = x4.z;
            x1[a + 3] = x4.w;
        }
    } else {
#pragma unroll
        for (int a = 0; a < W; ++a) x1[a] = x[a];
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t row = lane + 32u * r;
        if (row < Lay::top_rows) {
            // chains T^{D-1} (the new S_{D-1}) and T^D along the row's prefixes
            float accd = t1[D];
            float accm = t1[D - 1];
#pragma unroll
            for (int j = 2; j < D - 1; ++j) {
                const uint32_t pref = row / cpow(W, D - 1 - j);
                const float sj = S[Lay::s_off(j) + pref];
                const float xp = x[pref % W];
                accd = fmaf(accd, __fmul_rn(xp, 1.0f / static_cast<float>(D - j + 1)), sj);
                accm = fmaf(accm, __fmul_rn(xp, 1.0f / static_cast<float>(D - j)), sj);
            }
            if constexpr (Lay::reg_dm1) {
                const float xa = x[row % W];
                accd = fmaf(accd, __fmul_rn(xa, 0.5f), sd[r]);  // T^D_{D-1}: old S_{D-1}
                sd[r] = fmaf(accm, xa, sd[r]);       // new S_{D-1} = T^{D-1}_{D-1}
            }
#pragma unroll
            for (int a = 0; a < W; ++a) top[r][a] = fmaf(accd, x1[a], top[r][a]);
        }
    }
    __syncwarp();  // every lane has read the old levels
    v = 0;
    if (lane == 0) S[Lay::s_off(1)] = nv[0];
    ++v;
#pragma unroll
    for (int n = 2; n <= NS; ++n) {
        const uint32_t sl = Lay::slice(n);
#pragma unroll
        for (uint32_t q = 0; q < (sl + 31) / 32; ++q, ++v) {
            const uint32_t u = lane + 32u * q;
            if (u < sl) S[Lay::s_off(n) + u] = nv[v];
        }
    }
}

// One path b with increments [off, off + len) by warp c of the path's W
// warps (its first-letter slice), into the signature row sig + b*sig_stride.
// `region` is the warp's shared memory (LetterLayout::warp_floats floats:
// two increment buffers, then the levels kept in shared memory).  Warps
// never wait on each other; ends with __syncwarp.
template <int W, int D>
__device__ __forceinline__ void letter_path(const float* __restrict__ incr, int64_t b, int64_t off, int64_t len,
                                            float* sig, int64_t sig_stride, float* region, uint32_t c,
                                            uint32_t lane) {
    using Lay = LetterLayout<W, D>;
    static_assert(D >= 2 && W <= 32, "one letter per lane");
    static_assert(LetterLayout<W, D>::rows_per_lane * W <= 32, "at most 32 registers of top-level rows");
    constexpr int R = Lay::rows_per_lane;
    constexpr int PF = 8;  // increments prefetched ahead
    float* xcb = region;             // two increment buffers
    float* S = xcb + 2 * Lay::xcs;   // levels 1..smem_levels
    const bool xlane = lane < static_cast<uint32_t>(W);  // lane a < W holds letter a
    const float* xin = incr + off * W;
    for (uint32_t i = lane; i < Lay::s_size; i += 32) S[i] = 0.0f;
    float top[R][W];
    float sd[R];  // this lane's coefficients of level D-1 (when in registers)
#pragma unroll
    for (int i = 0; i < R; ++i) {
        sd[i] = 0.0f;
#pragma unroll
        for (int a = 0; a < W; ++a) top[i][a] = 0.0f;
    }
    // prefetch ring: xr[q] holds this lane's letter of increment k0 + q for
    // the block of PF steps starting at k0 (loads issued PF steps ahead, so
    // their L2 latency is hidden behind PF short steps)
    float xr[PF];
#pragma unroll
    for (int q = 0; q < PF; ++q) xr[q] = (xlane && q < len) ? __ldg(xin + q * W + lane) : 0.0f;
    if (xlane && len > 0) xcb[lane] = xr[0];
    __syncwarp();
    for (int64_t k0 = 0; k0 < len; k0 += PF) {
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            const int64_t k = k0 + q;
            if (k >= len) break;
            // slot q has been consumed (x_k is in the increment buffer):
            // refill it with x_{k+PF}
            if (xlane && k + PF < len) xr[q] = __ldg(xin + (k + PF) * W + lane);
            letter_step<W, D>(S, xcb + (k & 1) * Lay::xcs, top, sd, c, lane);
            if (xlane && k + 1 < len) xcb[((k + 1) & 1) * Lay::xcs + lane] = xr[(q + 1) % PF];
            __syncwarp();
        }
    }
    // the signature row: S_0 (warp 0), the slices of levels 1..D-1 and the
    // top rows
    float* dst = sig + b * sig_stride;
    if (c == 0 && lane == 0) dst[0] = 1.0f;
#pragma unroll
    for (int j = 1; j <= Lay::smem_levels; ++j) {
        const uint32_t sl = Lay::slice(j);
        for (uint32_t u = lane; u < sl; u += 32) dst[level_start<W>(j) + c * sl + u] = S[Lay::s_off(j) + u];
    }
    float* ddm1 = dst + level_start<W>(D - 1) + c * Lay::slice(D - 1);
    float* dtop = dst + level_start<W>(D) + c * Lay::slice(D);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t row = lane + 32u * r;
        if (row < Lay::top_rows) {
            if constexpr (Lay::reg_dm1) ddm1[row] = sd[r];
#pragma unroll
            for (int a = 0; a < W; ++a) dtop[row * W + a] = top[r][a];
        }
    }
    __syncwarp();
}

// The instantiated (width, depth) shapes, as X(width, depth) entries: at most
// 32 registers of top-level rows per lane, and few enough lower-level
// coefficients per lane to stay within 64 registers (W4 D6 and W3 D7 needed
// 168 in an earlier form).
#define RPP_GB_LETTER_SHAPES(X) \
    X(8, 2) X(8, 3) X(8, 4) X(5, 2) X(5, 3) X(5, 4) X(5, 5) X(4, 4) X(4, 5) X(6, 4) X(3, 5) X(3, 6) X(16, 2)

}  // namespace
}  // namespace rpp_gb
