// signature_letters.cuh -- FP32 signatures with one warp per first letter:
// the forward step (k_signature_letters in signature_fp32.cu, and FP32
// forward-only jobs of the grouped launch in signature_group.cu) and, below
// the forward part, the reverse step (k_signature_letters_rev).
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
//    two or three __syncwarp per step.  The one exception: the two chains
//    the top rows continue are formed once per level D-2 coefficient and
//    shared by its W top rows through shared memory.
//  * Width and depth are compile-time, so every stage, chain offset, level
//    size and index split is a constant and the loops unroll.
//  * The top level lives in registers: lane l holds the rows l, l + 32, ... of
//    the warp's slice (W coefficients sharing one prefix), so one chain value
//    serves W FMAs with the increment in registers.  No chain reads the top
//    level, so no other thread needs it.  Level D-1 lives in registers too:
//    lane l holds its coefficients l, l + 32, ..., which are exactly the
//    prefixes of its top rows and are read by no other lane.  Where level
//    D-2 has 24..32 coefficients per warp (W5 D5, W3 D6) the family form
//    gives lane u level D-2 coefficient u, its W children and their W^2 top
//    coefficients instead.
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
// registers; at D = 2 level 1 stays in shared memory), then (D >= 4) the two
// top-row chains of each level D-2 coefficient.  Each warp's region is a
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
    // Family form (letter_step_family): when level D-2 of a slice has 24..32
    // coefficients (W5 D5: 25, W3 D6: 27), lane u < fam holds level D-2
    // coefficient u, its W children on level D-1 and their W^2 top
    // coefficients in registers, so their chains are formed once per lane
    // with compile-time letters; levels 1..D-3 stay in shared memory.
    static constexpr uint32_t fam = D >= 4 ? slice(D - 2) : 0;
    static constexpr bool family = D >= 4 && fam >= 24 && fam <= 32;
    static constexpr int smem_levels = family ? D - 3 : reg_dm1 ? D - 2 : D - 1;
    static constexpr uint32_t s_size = s_off(smem_levels + 1);
    // D >= 4, row form: the chains T^{D-1} and T^D at each level D-2
    // coefficient, shared by the W top rows below it (after S: [0, W^{D-3})
    // and [W^{D-3}, 2 W^{D-3}))
    static constexpr bool shared_chains = D >= 4 && !family;
    static constexpr uint32_t cb_size = shared_chains ? 2 * slice(D - 2) : 0;
    static constexpr uint32_t xcs = (W + 3) / 4 * 4;       // one increment buffer (x_a)
    static constexpr uint32_t warp_floats = (2 * xcs + s_size + cb_size + 3) / 4 * 4;
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

// The W letters of an increment buffer into registers (16-byte loads when W
// is a multiple of 4; the buffers are 16-byte aligned).
template <int W>
__device__ __forceinline__ void load_letters(float (&x1)[W], const float* xb) {
    if constexpr (W % 4 == 0) {
#pragma unroll
        for (int a = 0; a < W; a += 4) {
            const float4 x4 = *reinterpret_cast<const float4*>(xb + a);
            x1[a] = x4.x;
            x1[a + 1] = x4.y;
            x1[a + 2] = x4.z;
            x1[a + 3] = x4.w;
        }
    } else {
#pragma unroll
        for (int a = 0; a < W; ++a) x1[a] = xb[a];
    }
}

// One forward step of warp c (its first-letter slice).  Every coefficient's
// Horner chain is evaluated by the lane that updates it, from the old lower
// levels: for a word (c, a_2, ..., a_n) of level n,
//     T_1 = S_1 + x_c / n,   T_j = S_j[a_1..a_j] + T_{j-1} x_{a_j} / (n-j+1),
// and the new S_n is T_n (the top level adds T_{D-1} x_a to its registers).
// These are the shared-memory kernel's chain values, formed by the same fused
// multiply-adds in the same order, so the results are identical; the sharing
// of a prefix's chain value between coefficients is given up on levels 1..D-2
// (their chains are short), for no chain arrays, no stage barriers and little
// index arithmetic.  The top rows' chains to level D-2 (D >= 4) are formed
// beside the level D-2 coefficient's own and read from shared memory by its W
// rows (one __syncwarp): recomputed per row they cost (D-3) loads, multiplies
// and FMAs twice over.  All lanes read the old levels before any lane writes
// the new ones (one __syncwarp between); the caller's __syncwarp after
// refreshing the increment orders the writes before the next step's reads.
// `with_top` false: the top rows are left alone (a gradient-only call needs
// levels 1..D-1 only).
template <int W, int D>
__device__ __forceinline__ void letter_step(float* S, const float* x,
                                            float (&top)[LetterLayout<W, D>::rows_per_lane][W],
                                            float (&sd)[LetterLayout<W, D>::rows_per_lane], uint32_t c,
                                            uint32_t lane, bool with_top = true) {
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
                // on level D-2 (D >= 4) also the chains T^D and T^{D-1} of u,
                // which the W top rows below u continue
                constexpr bool tops = Lay::shared_chains;
                float accd = t1[D], accm = t1[D - 1];
#pragma unroll
                for (int j = 2; j <= n; ++j) {
                    const uint32_t pref = u / cpow(W, n - j);  // index of (c, a_2..a_j) in level j's slice
                    const float xp = x[pref % W];
                    const float sj = S[Lay::s_off(j) + pref];
                    acc = fmaf(acc, __fmul_rn(xp, 1.0f / static_cast<float>(n - j + 1)), sj);
                    if (tops && n == NS) {
                        accd = fmaf(accd, __fmul_rn(xp, 1.0f / static_cast<float>(D - j + 1)), sj);
                        accm = fmaf(accm, __fmul_rn(xp, 1.0f / static_cast<float>(D - j)), sj);
                    }
                }
                nv[v] = acc;
                if (tops && n == NS) {
                    S[Lay::s_size + u] = accm;
                    S[Lay::s_size + sl + u] = accd;
                }
            }
        }
    }
    if constexpr (Lay::shared_chains) __syncwarp();  // the top rows' chains are in place
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
            // chains T^{D-1} (the new S_{D-1}) and T^D along the row's
            // prefixes, to level D-2: from the level D-2 pass (D >= 4)
            float accd = t1[D];
            float accm = t1[D - 1];
            if constexpr (Lay::shared_chains) {
                accm = S[Lay::s_size + row / W];
                accd = S[Lay::s_size + Lay::slice(D - 2) + row / W];
            }
            if constexpr (Lay::reg_dm1) {
                const float xa = x[row % W];
                accd = fmaf(accd, __fmul_rn(xa, 0.5f), sd[r]);  // T^D_{D-1}: old S_{D-1}
                sd[r] = fmaf(accm, xa, sd[r]);       // new S_{D-1} = T^{D-1}_{D-1}
            }
            if (with_top) {
#pragma unroll
                for (int a = 0; a < W; ++a) top[r][a] = fmaf(accd, x1[a], top[r][a]);
            }
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

// One forward step of warp c, family form (LetterLayout::family): levels
// 1..D-3 as in letter_step; lane u < fam forms the chains of its level D-2
// coefficient u along u's prefixes (to T^{D-2}, the new S_{D-2}[u], and the
// chains T^{D-1}, T^D its children continue), then its W children on level
// D-1 and their top rows with compile-time letters.  The same fused
// multiply-adds in the same order as letter_step, so the results are
// identical.
template <int W, int D>
__device__ __forceinline__ void letter_step_family(float* S, const float* x, float (&top)[W][W], float (&sdf)[W],
                                                   float& sf, uint32_t c, uint32_t lane, bool with_top) {
    using Lay = LetterLayout<W, D>;
    constexpr int NS = Lay::smem_levels;  // D - 3 >= 1
    const float s1 = S[Lay::s_off(1)];
    const float xcc = x[c];
    float t1[D + 1];  // T^n_1 = S_1 + S_0 x_c / n (S_0 = 1)
#pragma unroll
    for (int n = 2; n <= D; ++n) t1[n] = s1 + __fmul_rn(xcc, 1.0f / static_cast<float>(n));
    float nv[lower_per_lane<W, D>() > 0 ? lower_per_lane<W, D>() : 1];
    int v = 0;
    nv[v++] = s1 + xcc;
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
                    const uint32_t pref = u / cpow(W, n - j);
                    acc = fmaf(acc, __fmul_rn(x[pref % W], 1.0f / static_cast<float>(n - j + 1)),
                               S[Lay::s_off(j) + pref]);
                }
                nv[v] = acc;
            }
        }
    }
    float x1[W];
    load_letters<W>(x1, x);
    if (lane < Lay::fam) {
        const uint32_t u = lane;
        float acc = t1[D - 2], accm = t1[D - 1], accd = t1[D];
#pragma unroll
        for (int j = 2; j <= D - 2; ++j) {
            const uint32_t pref = u / cpow(W, D - 2 - j);
            const float xp = x[pref % W];
            const float sj = j == D - 2 ? sf : S[Lay::s_off(j) + pref];
            acc = fmaf(acc, __fmul_rn(xp, 1.0f / static_cast<float>(D - 2 - j + 1)), sj);
            accd = fmaf(accd, __fmul_rn(xp, 1.0f / static_cast<float>(D - j + 1)), sj);
            accm = fmaf(accm, __fmul_rn(xp, 1.0f / static_cast<float>(D - j)), sj);
        }
        sf = acc;
#pragma unroll
        for (int a = 0; a < W; ++a) {
            const float ad = fmaf(accd, __fmul_rn(x1[a], 0.5f), sdf[a]);  // T^D_{D-1}: old S_{D-1}
            sdf[a] = fmaf(accm, x1[a], sdf[a]);                            // new S_{D-1}
            if (with_top) {
#pragma unroll
                for (int e = 0; e < W; ++e) top[a][e] = fmaf(ad, x1[e], top[a][e]);
            }
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

// The increment loop of one path's forward pass by one warp: lane a < W
// loads letter a eight steps ahead into a register ring (a step here is
// short, and a load one step ahead left the L2 latency exposed); `step(x)`
// runs each step on the increment buffer x (two buffers by step parity in
// xcb).  Ends with __syncwarp.
template <int W, int D, typename Step>
__device__ __forceinline__ void letter_forward_loop(const float* __restrict__ incr, int64_t off, int64_t len,
                                                    float* xcb, uint32_t lane, Step&& step) {
    using Lay = LetterLayout<W, D>;
    constexpr int PF = 8;  // increments prefetched ahead
    const bool xlane = lane < static_cast<uint32_t>(W);  // lane a < W holds letter a
    const float* xin = incr + off * W;
    // xr[q] holds this lane's letter of increment k0 + q for the block of PF
    // steps starting at k0
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
            step(xcb + (k & 1) * Lay::xcs);
            if (xlane && k + 1 < len) xcb[((k + 1) & 1) * Lay::xcs + lane] = xr[(q + 1) % PF];
            __syncwarp();
        }
    }
}

// The forward pass of one path with increments [off, off + len) by warp c of
// the path's W warps (its first-letter slice), row form: leaves levels
// 1..smem_levels of the slice in S, level D-1 in sd and, with `with_top`, the
// top rows in `top`.  `xcb` holds the two increment buffers (2 xcs floats).
// Warps never wait on each other; ends with __syncwarp.
template <int W, int D>
__device__ __forceinline__ void letter_forward(const float* __restrict__ incr, int64_t off, int64_t len, float* xcb,
                                               float* S, float (&top)[LetterLayout<W, D>::rows_per_lane][W],
                                               float (&sd)[LetterLayout<W, D>::rows_per_lane], uint32_t c,
                                               uint32_t lane, bool with_top) {
    using Lay = LetterLayout<W, D>;
    static_assert(D >= 2 && W <= 32, "one letter per lane");
    static_assert(LetterLayout<W, D>::rows_per_lane * W <= 32, "at most 32 registers of top-level rows");
    constexpr int R = Lay::rows_per_lane;
    for (uint32_t i = lane; i < Lay::s_size; i += 32) S[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < R; ++i) {
        sd[i] = 0.0f;
#pragma unroll
        for (int a = 0; a < W; ++a) top[i][a] = 0.0f;
    }
    letter_forward_loop<W, D>(incr, off, len, xcb, lane,
                              [&](const float* x) { letter_step<W, D>(S, x, top, sd, c, lane, with_top); });
}

// The same, family form (LetterLayout::family): lane u < fam ends with level
// D-2 coefficient u in sf, its children's level D-1 coefficients in sdf and,
// with `with_top`, their top rows in `top`.
template <int W, int D>
__device__ __forceinline__ void letter_forward_family(const float* __restrict__ incr, int64_t off, int64_t len,
                                                      float* xcb, float* S, float (&top)[W][W], float (&sdf)[W],
                                                      float& sf, uint32_t c, uint32_t lane, bool with_top) {
    using Lay = LetterLayout<W, D>;
    static_assert(Lay::family, "family form");
    for (uint32_t i = lane; i < Lay::s_size; i += 32) S[i] = 0.0f;
    sf = 0.0f;
#pragma unroll
    for (int i = 0; i < W; ++i) {
        sdf[i] = 0.0f;
#pragma unroll
        for (int a = 0; a < W; ++a) top[i][a] = 0.0f;
    }
    letter_forward_loop<W, D>(incr, off, len, xcb, lane, [&](const float* x) {
        letter_step_family<W, D>(S, x, top, sdf, sf, c, lane, with_top);
    });
}

// Warp c's part of the signature row dst: S_0 (warp 0), the slices of levels
// 1..D-1 and the top rows.
template <int W, int D>
__device__ __forceinline__ void letter_store(float* dst, const float* S,
                                             const float (&top)[LetterLayout<W, D>::rows_per_lane][W],
                                             const float (&sd)[LetterLayout<W, D>::rows_per_lane], uint32_t c,
                                             uint32_t lane) {
    using Lay = LetterLayout<W, D>;
    constexpr int R = Lay::rows_per_lane;
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
}

// The same, family form: levels 1..D-3 from S, then lane u < fam's level D-2
// coefficient, its children's level D-1 coefficients and their top rows.
template <int W, int D>
__device__ __forceinline__ void letter_store_family(float* dst, const float* S, const float (&top)[W][W],
                                                    const float (&sdf)[W], float sf, uint32_t c, uint32_t lane) {
    using Lay = LetterLayout<W, D>;
    if (c == 0 && lane == 0) dst[0] = 1.0f;
#pragma unroll
    for (int j = 1; j <= Lay::smem_levels; ++j) {
        const uint32_t sl = Lay::slice(j);
        for (uint32_t u = lane; u < sl; u += 32) dst[level_start<W>(j) + c * sl + u] = S[Lay::s_off(j) + u];
    }
    if (lane < Lay::fam) {
        const uint32_t u = lane;
        dst[level_start<W>(D - 2) + c * Lay::slice(D - 2) + u] = sf;
        float* ddm1 = dst + level_start<W>(D - 1) + c * Lay::slice(D - 1) + u * W;
        float* dtop = dst + level_start<W>(D) + c * Lay::slice(D) + u * W * W;
#pragma unroll
        for (int a = 0; a < W; ++a) {
            ddm1[a] = sdf[a];
#pragma unroll
            for (int e = 0; e < W; ++e) dtop[a * W + e] = top[a][e];
        }
    }
}

// One path b with increments [off, off + len) by warp c of the path's W
// warps, into the signature row sig + b*sig_stride.  `region` is the warp's
// shared memory (LetterLayout::warp_floats floats: two increment buffers,
// then the levels kept in shared memory).  Ends with __syncwarp.
template <int W, int D>
__device__ __forceinline__ void letter_path(const float* __restrict__ incr, int64_t b, int64_t off, int64_t len,
                                            float* sig, int64_t sig_stride, float* region, uint32_t c,
                                            uint32_t lane) {
    using Lay = LetterLayout<W, D>;
    float* S = region + 2 * Lay::xcs;
    if constexpr (Lay::family) {
        float top[W][W], sdf[W], sf;
        letter_forward_family<W, D>(incr, off, len, region, S, top, sdf, sf, c, lane, true);
        letter_store_family<W, D>(sig + b * sig_stride, S, top, sdf, sf, c, lane);
    } else {
        constexpr int R = Lay::rows_per_lane;
        float top[R][W];
        float sd[R];
        letter_forward<W, D>(incr, off, len, region, S, top, sd, c, lane, true);
        letter_store<W, D>(sig + b * sig_stride, S, top, sd, c, lane);
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// Reverse mode with one warp per first letter (k_signature_letters_rev).
//
// The reverse step of signature_body.cuh restated on first-letter slices.
// For increment x = x_k, S = S_k and the cotangent G' = G_k of S_k:
//  * Recovery: S_{k-1} follows from S_k level by level, bottom-up, by undoing
//    the forward Horner chains: S^-_j[u] = S_j[u] - T^j_{j-1}[p] x_a for
//    u = (p, a), and the chains of the recovered state,
//    T^n_j[u] = S^-_j[u] + T^n_{j-1}[p] x_a / (n-j+1) (T^n_0 = 1).
//  * Cotangent chains, top-down: A^n_n = G'_n and
//    A^n_{j-1}[p] = sum_a A^n_j[p a] x_a / (n-j+1); G_{k-1,j} = sum_{n>=j} A^n_j
//    (the top level of G never changes).
//  * Letter gradient: xbar_a = sum_{n, j, p} A^n_j[p a] T^n_{j-1}[p] / (n-j+1).
// Every term of a word's chains involves only its prefixes, which share its
// first letter, so warp c runs the step on its slice alone; only the letter
// gradient sums over all slices (a butterfly in the warp, then W warps'
// partials added in warp order once per 8 steps, after one CTA barrier).
// Shared-memory instructions bounded the first form of this kernel (with the
// lower levels of S and G and a table of x_a / m in shared memory), so
// everything a lane alone reads lives in its registers: the seed's top rows
// (constant through the pass), and of S and G level D-1 (lane l: rows l,
// l + 32, ...) and the lane's own coefficients of levels 1..D-2 (l, l + 32,
// ... of each level); the family form (LetterRevLayout::family) regroups
// levels D-2..D by families.
// Scaled increments x_a / m are formed in registers (x_a * (1/m), rounded
// once).  Shared memory holds only what other lanes read: the increment, the
// chains T^n_j of levels 1..D-2 and the cotangent chains A^n_j of levels
// 1..D-1.  A step has 2D-2 warp barriers and no CTA barrier: recovery passes
// for levels 1..D-2; the top rows (the recovery of level D-1, A^D_{D-1} and
// the top level's letter terms); per level j = D-2..1 a pass over the
// (chain n, row p) pairs (A^n_j[p] and the letter terms of p's children);
// and one that updates G on levels 1..D-2.
template <int W, int D>
struct LetterRevLayout {
    using F = LetterLayout<W, D>;
    static_assert(D >= 3, "level D-1 in registers");
    static constexpr uint32_t sl(int j) { return F::slice(j); }
    static constexpr uint32_t xb_off = F::warp_floats;  // two increment buffers, by step parity
    static constexpr uint32_t tf_off = xb_off + 2 * F::xcs;
    // level j (1..D-2): T^n_j for n = j+1..D
    static constexpr uint32_t tf_rel(int j) {
        uint32_t o = 0;
        for (int i = 1; i < j; ++i) o += (D - i) * sl(i);
        return o;
    }
    static constexpr uint32_t tf(int j, int n) { return tf_off + tf_rel(j) + (n - j - 1) * sl(j); }
    // level j (1..D-1): A^n_j for n = j..D (A^j_j: the old G_j)
    static constexpr uint32_t ab_off = tf_off + tf_rel(D - 1);
    static constexpr uint32_t ab_rel(int j) {
        uint32_t o = 0;
        for (int i = 1; i < j; ++i) o += (D - i + 1) * sl(i);
        return o;
    }
    static constexpr uint32_t ab(int j, int n) { return ab_off + ab_rel(j) + (n - j) * sl(j); }
    static constexpr uint32_t warp_floats = (ab_off + ab_rel(D) + 3) / 4 * 4;
    // registers: the lane's coefficients of levels 1..D-2 (lo), and the
    // scale 1 / (n - j) of each (chain n, row) pair the lane takes (pr)
    static constexpr int lo(int j) {
        int o = 0;
        for (int i = 1; i < j; ++i) o += static_cast<int>((sl(i) + 31) / 32);
        return o;
    }
    static constexpr int pr(int j) {
        int o = 0;
        for (int i = 1; i < j; ++i) o += static_cast<int>(((D - i) * sl(i) + 31) / 32);
        return o;
    }
    static constexpr int lo_total = lo(D - 1) > 0 ? lo(D - 1) : 1;
    static constexpr int pr_total = pr(D - 1) > 0 ? pr(D - 1) : 1;
    // Family form (letter_reverse_step_family): when level D-2 of a slice has
    // 24..32 coefficients (W5 D5: 25, W3 D6: 27), lane u < fam owns level D-2
    // coefficient u, its W children on level D-1 and their W^2 top
    // coefficients, so the recovery of level D-1, the top rows and the
    // cotangent chains of level D-2 run in its registers with compile-time
    // letters; only levels 1..D-3 go through the passes over shared memory.
    static constexpr uint32_t fam = F::fam;
    static constexpr bool family = F::family;
    static constexpr int lower = family ? D - 3 : D - 2;  // levels of the shared-memory passes
    static constexpr int steps_per_block = 8;  // letter partials reduced across warps once per block
    // per CTA after the W warp regions: [2][steps_per_block][W warps][W letters]
    static constexpr uint32_t pbuf_floats = 2u * steps_per_block * W * W;
};

// Recovery of levels 1..LL of warp c's slice, bottom-up, with their chains
// (the lane's coefficients in slo).  Ends with __syncwarp.
template <int W, int D, int LL>
__device__ __forceinline__ void letter_recover_lower(float* region, const float* xb,
                                                     float (&slo)[LetterRevLayout<W, D>::lo_total], uint32_t c,
                                                     uint32_t lane) {
    using F = LetterLayout<W, D>;
    using Rev = LetterRevLayout<W, D>;
#pragma unroll
    for (int j = 1; j <= LL; ++j) {
        const uint32_t sl = F::slice(j);
#pragma unroll
        for (uint32_t q = 0; q < (sl + 31) / 32; ++q) {
            const uint32_t u = lane + 32u * q;
            if (u < sl) {
                const uint32_t a = j == 1 ? c : u % W;
                const uint32_t p = u / W;  // the prefix, in level j-1's slice (j >= 2)
                const float xv = xb[a];
                const float s = fmaf(j == 1 ? -1.0f : -region[Rev::tf(j - 1, j) + p], xv, slo[Rev::lo(j) + q]);
                slo[Rev::lo(j) + q] = s;
#pragma unroll
                for (int n = j + 1; n <= D; ++n) {
                    const float par = j == 1 ? 1.0f : region[Rev::tf(j - 1, n) + p];
                    region[Rev::tf(j, n) + u] = fmaf(par, __fmul_rn(xv, 1.0f / static_cast<float>(n - j + 1)), s);
                }
            }
        }
        __syncwarp();
    }
}

// Levels LL..1: the cotangent chains of each (chain n, row p) pair from p's
// children on level j+1 (chain n = j+1: G_{j+1} as of the step's start),
// with the children's letter terms; then G_j += sum_{n>j} A^n_j on levels
// 1..LL (the lane's own coefficients), the new value copied to chain n = j
// of level j for the next step's pass over level j-1, and the letter term of
// the word c, sum_n A^n_1 / n with A^1_1 the old G_1.  Ends with __syncwarp.
template <int W, int D, int LL>
__device__ __forceinline__ void letter_cotangent_lower(float* region, const float (&x1)[W],
                                                       float (&glo)[LetterRevLayout<W, D>::lo_total],
                                                       const float (&pinv)[LetterRevLayout<W, D>::pr_total],
                                                       float (&xa)[W], uint32_t c, uint32_t lane) {
    using F = LetterLayout<W, D>;
    using Rev = LetterRevLayout<W, D>;
#pragma unroll
    for (int j = LL; j >= 1; --j) {
        const uint32_t sl = F::slice(j);
        const uint32_t pairs = static_cast<uint32_t>(D - j) * sl;
#pragma unroll
        for (uint32_t q = 0; q < (pairs + 31) / 32; ++q) {
            const uint32_t e = lane + 32u * q;  // (n - j - 1) sl + p
            if (e < pairs) {
                const float inv = pinv[Rev::pr(j) + q];                     // 1 / (n - j)
                const float* ch = region + Rev::ab(j + 1, j + 1) + W * e;  // A^n_{j+1}[p a], a = 0..W-1
                const float tx = __fmul_rn(region[Rev::tf(j, j + 1) + e], inv);  // T^n_j[p] / (n - j)
                float acc = 0.0f;
#pragma unroll
                for (int a = 0; a < W; ++a) {
                    const float g = ch[a];
                    acc = fmaf(g, __fmul_rn(x1[a], inv), acc);
                    xa[a] = fmaf(g, tx, xa[a]);
                }
                region[Rev::ab(j, j) + sl + e] = acc;  // A^n_j[p]
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int j = 1; j <= LL; ++j) {
        const uint32_t sl = F::slice(j);
#pragma unroll
        for (uint32_t q = 0; q < (sl + 31) / 32; ++q) {
            const uint32_t u = lane + 32u * q;
            if (u < sl) {
                float g = glo[Rev::lo(j) + q];
                float term = g;
#pragma unroll
                for (int n = j + 1; n <= D; ++n) {
                    const float an = region[Rev::ab(j, n) + u];
                    g += an;
                    if (j == 1) term = fmaf(an, 1.0f / static_cast<float>(n), term);
                }
                glo[Rev::lo(j) + q] = g;
                region[Rev::ab(j, j) + u] = g;
                if (j == 1) {
#pragma unroll
                    for (int a = 0; a < W; ++a)
                        if (static_cast<uint32_t>(a) == c) xa[a] += term;
                }
            }
        }
    }
    __syncwarp();
}


// One reverse step of warp c, row form.  `region` is the warp's shared
// memory, `xb` the step's increment (x_a at a).  sd / gd: levels D-1 of S and
// G (rows lane + 32 q); slo / glo: the lane's coefficients of levels 1..D-2;
// pinv: its pair scales.  Adds this warp's letter terms to xa.  Ends with
// __syncwarp.
template <int W, int D>
__device__ __forceinline__ void letter_reverse_step(float* region, const float* xb,
                                                    const float (&gtop)[LetterLayout<W, D>::rows_per_lane][W],
                                                    float (&sd)[LetterLayout<W, D>::rows_per_lane],
                                                    float (&gd)[LetterLayout<W, D>::rows_per_lane],
                                                    float (&slo)[LetterRevLayout<W, D>::lo_total],
                                                    float (&glo)[LetterRevLayout<W, D>::lo_total],
                                                    const float (&pinv)[LetterRevLayout<W, D>::pr_total],
                                                    float (&xa)[W], uint32_t c, uint32_t lane) {
    using F = LetterLayout<W, D>;
    using Rev = LetterRevLayout<W, D>;
    constexpr int R = F::rows_per_lane;
    letter_recover_lower<W, D, D - 2>(region, xb, slo, c, lane);
    // the top rows: recovery of level D-1 (registers), T^D_{D-1}, A^D_{D-1}
    // and the top level's letter terms
    float x1[W];
    load_letters<W>(x1, xb);
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const uint32_t p = lane + 32u * q;
        if (p < F::top_rows) {
            const uint32_t pu = p / W, a = p % W;
            const float xl = xb[a];
            const float s = fmaf(-region[Rev::tf(D - 2, D - 1) + pu], xl, sd[q]);
            sd[q] = s;
            const float td = fmaf(region[Rev::tf(D - 2, D) + pu], __fmul_rn(xl, 0.5f), s);
            float acc = 0.0f;
#pragma unroll
            for (int e = 0; e < W; ++e) {
                acc = fmaf(gtop[q][e], x1[e], acc);
                xa[e] = fmaf(gtop[q][e], td, xa[e]);
            }
            region[Rev::ab(D - 1, D - 1) + p] = gd[q];
            region[Rev::ab(D - 1, D) + p] = acc;
            gd[q] += acc;
        }
    }
    __syncwarp();
    letter_cotangent_lower<W, D, D - 2>(region, x1, glo, pinv, xa, c, lane);
}

// One reverse step of warp c, family form (LetterRevLayout::family): lane
// u < fam holds level D-2 coefficient u of S and G (sf, gf), its children's
// level D-1 coefficients (sdf, gdf) and their top rows (gtop[a][b] = G'_D at
// (u, a, b)).  The family pass recovers u and its children, forms the top
// level's letter terms and A^D_{D-1} of each child, the children's letter
// terms on level D-1 and A^{D-1}_{D-2}, A^D_{D-2} of u -- the sums the row
// form spreads over its top pass and a pass over level D-2's pairs.  Ends
// with __syncwarp.
template <int W, int D>
__device__ __forceinline__ void letter_reverse_step_family(float* region, const float* xb, const float (&gtop)[W][W],
                                                           float (&sdf)[W], float (&gdf)[W], float& sf, float& gf,
                                                           float (&slo)[LetterRevLayout<W, D>::lo_total],
                                                           float (&glo)[LetterRevLayout<W, D>::lo_total],
                                                           const float (&pinv)[LetterRevLayout<W, D>::pr_total],
                                                           float (&xa)[W], uint32_t c, uint32_t lane) {
    using Rev = LetterRevLayout<W, D>;
    static_assert(Rev::family, "family form");
    letter_recover_lower<W, D, D - 3>(region, xb, slo, c, lane);
    float x1[W];
    load_letters<W>(x1, xb);
    if (lane < Rev::fam) {
        const uint32_t u = lane, pu = u / W;
        const float xv = xb[u % W];
        // recovery of u and its chains T^{D-1}_{D-2}, T^D_{D-2}
        const float s = fmaf(-region[Rev::tf(D - 3, D - 2) + pu], xv, sf);
        sf = s;
        const float tm = fmaf(region[Rev::tf(D - 3, D - 1) + pu], __fmul_rn(xv, 0.5f), s);
        const float td = fmaf(region[Rev::tf(D - 3, D) + pu], __fmul_rn(xv, 1.0f / 3.0f), s);
        const float td2 = __fmul_rn(td, 0.5f);  // T^D_{D-2}[u] / 2
        float am = 0.0f, ad = 0.0f;             // A^{D-1}_{D-2}[u], A^D_{D-2}[u]
#pragma unroll
        for (int a = 0; a < W; ++a) {
            const float xh = __fmul_rn(x1[a], 0.5f);
            const float s4 = fmaf(-tm, x1[a], sdf[a]);  // S^-_{D-1}[u a]
            sdf[a] = s4;
            const float t4 = fmaf(td, xh, s4);  // T^D_{D-1}[u a]
            float acc = 0.0f;                   // A^D_{D-1}[u a]
#pragma unroll
            for (int e = 0; e < W; ++e) {
                acc = fmaf(gtop[a][e], x1[e], acc);
                xa[e] = fmaf(gtop[a][e], t4, xa[e]);
            }
            const float go = gdf[a];  // A^{D-1}_{D-1}[u a]: the old G_{D-1}
            gdf[a] = go + acc;
            xa[a] = fmaf(go, tm, xa[a]);
            xa[a] = fmaf(acc, td2, xa[a]);
            am = fmaf(go, x1[a], am);
            ad = fmaf(acc, xh, ad);
        }
        region[Rev::ab(D - 2, D - 2) + u] = gf;
        region[Rev::ab(D - 2, D - 1) + u] = am;
        region[Rev::ab(D - 2, D) + u] = ad;
        gf = gf + am + ad;
    }
    __syncwarp();
    letter_cotangent_lower<W, D, D - 3>(region, x1, glo, pinv, xa, c, lane);
}

// The reverse loop of one path by warp c of team `tm` (the CTA, or a team of
// W warps of the grouped launch): increments from the last (lane a < W loads
// letter a four steps ahead), `step(xb, xa)` per increment, the warp's letter
// partials per step into pbuf, and once per 8 steps (and at the end) one team
// barrier after which ranks t < 8 W add the W warps' partials in warp order
// into the gradient rows.
template <int W, int D, typename Team, typename Step>
__device__ __forceinline__ void letter_reverse_loop(const Team& tm, const float* __restrict__ incr, int64_t off,
                                                    int64_t len, float* grad, float* region, float* pbuf, uint32_t c,
                                                    uint32_t lane, Step&& step) {
    using F = LetterLayout<W, D>;
    using Rev = LetterRevLayout<W, D>;
    constexpr int NB = Rev::steps_per_block;  // steps per partials block
    constexpr int PF = 4;                     // increments prefetched ahead = steps per loop iteration
    const bool xlane = lane < static_cast<uint32_t>(W);
    const float* xin = incr + off * W;
    float* xbuf = region + Rev::xb_off;
    float* gout = grad + off * W;
    float xr[PF];
#pragma unroll
    for (int q = 0; q < PF; ++q) xr[q] = (xlane && q < len) ? __ldg(xin + (len - 1 - q) * W + lane) : 0.0f;
    if (xlane && len > 0) xbuf[lane] = xr[0];
    __syncwarp();
    float xa[W];
#pragma unroll
    for (int a = 0; a < W; ++a) xa[a] = 0.0f;
    constexpr uint32_t halvings = W <= 1 ? 0u : W <= 2 ? 1u : W <= 4 ? 2u : W <= 8 ? 3u : 4u;
    for (int64_t i0 = 0; i0 < len; i0 += PF) {
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            const int64_t i = i0 + q;  // reverse step i: increment len - 1 - i
            if (i >= len) break;
            // ring slot q held increment i (now in the buffer): refill it
            // with increment i + PF
            if (xlane && i + PF < len) xr[q] = __ldg(xin + (len - 1 - i - PF) * W + lane);
            step(xbuf + (i & 1) * F::xcs, xa);
            if (xlane && i + 1 < len) xbuf[((i + 1) & 1) * F::xcs + lane] = xr[(q + 1) % PF];
            const uint32_t slot = static_cast<uint32_t>(i % NB);
            float* pb = pbuf + ((i / NB) & 1) * (NB * W * W);
            // this warp's letter partials: pb[slot][c][a]
            uint32_t base = 0, cnt = W;
            letter_butterfly<float, W>(xa, lane, 16u, base, cnt);
            if (cnt > 0u && (lane & ((32u >> halvings) - 1u)) == 0u) pb[(slot * W + c) * W + base] = xa[0];
#pragma unroll
            for (int a = 0; a < W; ++a) xa[a] = 0.0f;
            __syncwarp();
            if (slot == NB - 1 || i == len - 1) {
                // the block's gradient rows: the W warps' partials added in
                // warp order (the other half of pbuf takes the next block)
                tm.sync();
                const uint32_t t = tm.rank();
                if (t < (slot + 1) * W) {
                    const uint32_t st = t / W, a = t % W;
                    float v = 0.0f;
#pragma unroll
                    for (int w = 0; w < W; ++w) v += pb[(st * W + w) * W + a];
                    gout[(len - 1 - (i - slot + st)) * W + a] = v;
                }
            }
        }
    }
}

// Forward and reverse pass of one path by warp c of team `tm` (the CTA in
// k_signature_letters_rev, a team of W warps in the grouped launch).  Modes:
// kForward | kBackward [| kTopLevel] (the forward pass first, writing the
// signature row with kTopLevel) and kBackward | kLoadFinal (the final
// signature read from sig).  `pbuf` is the team's partials buffer
// (LetterRevLayout::pbuf_floats), `region` the warp's shared memory
// (LetterRevLayout::warp_floats).  Contains team barriers: every warp of the
// team runs the same path.
template <int W, int D, typename Team>
__device__ __forceinline__ void letter_fwd_bwd(const Team& tm, const float* __restrict__ incr, int64_t b, int64_t off,
                                               int64_t len, float* sig, int64_t sig_stride,
                                               const float* __restrict__ seed, int64_t seed_stride, float* grad,
                                               int mode, float* region, float* pbuf, uint32_t c, uint32_t lane) {
    using F = LetterLayout<W, D>;
    using Rev = LetterRevLayout<W, D>;
    constexpr int R = F::rows_per_lane;
    constexpr int LL = Rev::lower;
    float* S = region + 2 * F::xcs;
    const float* src = sig + b * sig_stride;
    const float* sdr = seed + b * seed_stride;
    const bool load = mode & kLoadFinal;
    const bool with_top = mode & kTopLevel;
    // the final state: level D-1 (and in the family form level D-2) in the
    // form's registers, levels 1..LL in S (forward pass) or from sig
    float sd[F::family ? 1 : R];
    float sdf[F::family ? W : 1], sf = 0.0f;
    if constexpr (F::family) {
        const bool fl = lane < Rev::fam;
        const uint32_t u = lane;
        if (load) {
#pragma unroll
            for (int a = 0; a < W; ++a) sdf[a] = fl ? src[level_start<W>(D - 1) + c * F::slice(D - 1) + u * W + a] : 0.0f;
            sf = fl ? src[level_start<W>(D - 2) + c * F::slice(D - 2) + u] : 0.0f;
        } else {
            float top[W][W];
            letter_forward_family<W, D>(incr, off, len, region, S, top, sdf, sf, c, lane, with_top);
            if (with_top && sig) letter_store_family<W, D>(sig + b * sig_stride, S, top, sdf, sf, c, lane);
        }
    } else {
        if (load) {
#pragma unroll
            for (int q = 0; q < R; ++q) {
                const uint32_t p = lane + 32u * q;
                sd[q] = p < F::top_rows ? src[level_start<W>(D - 1) + c * F::slice(D - 1) + p] : 0.0f;
            }
        } else {
            float top[R][W];
            letter_forward<W, D>(incr, off, len, region, S, top, sd, c, lane, with_top);
            if (with_top && sig) letter_store<W, D>(sig + b * sig_stride, S, top, sd, c, lane);
        }
    }
    float slo[Rev::lo_total], glo[Rev::lo_total];
#pragma unroll
    for (int j = 1; j <= LL; ++j)
#pragma unroll
        for (uint32_t q = 0; q < (F::slice(j) + 31) / 32; ++q) {
            const uint32_t u = lane + 32u * q;
            const bool own = u < F::slice(j);
            slo[Rev::lo(j) + q] = !own ? 0.0f : load ? src[level_start<W>(j) + c * F::slice(j) + u] : S[F::s_off(j) + u];
            glo[Rev::lo(j) + q] = own ? sdr[level_start<W>(j) + c * F::slice(j) + u] : 0.0f;
            // chain n = j of level j: G_j as of the first step's start
            if (own) region[Rev::ab(j, j) + u] = glo[Rev::lo(j) + q];
        }
    // the scale 1 / (n - j) of each (chain n, row) pair of level j this lane
    // takes: pair e = lane + 32 q, n - j = e / W^{j-1} + 1
    float pinv[Rev::pr_total];
#pragma unroll
    for (int j = 1; j <= LL; ++j)
#pragma unroll
        for (uint32_t q = 0; q < ((D - j) * F::slice(j) + 31) / 32; ++q)
            pinv[Rev::pr(j) + q] = 1.0f / static_cast<float>((lane + 32u * q) / F::slice(j) + 1);
    if constexpr (Rev::family) {
        const uint32_t u = lane;
        const bool fl = u < Rev::fam;
        float gdf[W], gtop[W][W];
#pragma unroll
        for (int a = 0; a < W; ++a) {
            gdf[a] = fl ? sdr[level_start<W>(D - 1) + c * F::slice(D - 1) + u * W + a] : 0.0f;
#pragma unroll
            for (int e = 0; e < W; ++e)
                gtop[a][e] = fl ? sdr[level_start<W>(D) + c * F::slice(D) + (u * W + a) * W + e] : 0.0f;
        }
        float gf = fl ? sdr[level_start<W>(D - 2) + c * F::slice(D - 2) + u] : 0.0f;
        letter_reverse_loop<W, D>(tm, incr, off, len, grad, region, pbuf, c, lane, [&](const float* xb, float(&xa)[W]) {
            letter_reverse_step_family<W, D>(region, xb, gtop, sdf, gdf, sf, gf, slo, glo, pinv, xa, c, lane);
        });
    } else {
        float gtop[R][W], gd[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const uint32_t p = lane + 32u * q;
            const bool row = p < F::top_rows;
            gd[q] = row ? sdr[level_start<W>(D - 1) + c * F::slice(D - 1) + p] : 0.0f;
#pragma unroll
            for (int a = 0; a < W; ++a)
                gtop[q][a] = row ? sdr[level_start<W>(D) + c * F::slice(D) + p * W + a] : 0.0f;
        }
        letter_reverse_loop<W, D>(tm, incr, off, len, grad, region, pbuf, c, lane, [&](const float* xb, float(&xa)[W]) {
            letter_reverse_step<W, D>(region, xb, gtop, sd, gd, slo, glo, pinv, xa, c, lane);
        });
    }
}

// The instantiated (width, depth) shapes, as X(width, depth) entries: at most
// 32 registers of top-level rows per lane, and few enough lower-level
// coefficients per lane to stay within 64 registers (W4 D6 and W3 D7 needed
// 168 in an earlier form).
#define RPP_GB_LETTER_SHAPES(X) \
    X(8, 2) X(8, 3) X(8, 4) X(5, 2) X(5, 3) X(5, 4) X(5, 5) X(4, 4) X(4, 5) X(6, 4) X(3, 5) X(3, 6) X(16, 2)

}  // namespace
}  // namespace rpp_gb
