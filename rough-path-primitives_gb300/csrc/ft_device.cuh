// ft_device.cuh -- device building blocks shared by the per-operation kernels
// (ft_ops.cu) and the fused Lie <-> tensor kernels (lie_fused.cu): level-wise
// products over degree-range operands and the Horner intermediates
// (exp / fmexp / log) on a work buffer in shared or global memory.
#pragma once

#include "common.cuh"
#include "ops.hpp"

namespace rpp_gb {
namespace ftdev {

template <typename T>
struct Opnd {
    const T* p;
    int lo;
    int hi;
};

// Pipelined: the next split's index and operands are fetched before this
// split's FMA (same FMAs in the same order) -- faster for the Horner
// intermediates (ft_log, W5 D5: 0.232 -> 0.215 ms), slower for the plain
// products (ft_mul, W4 D4: 7.9 -> 9.4 us per launch), which keep the simple loop.
template <bool Pipelined, typename T>
__device__ __forceinline__ T split_sum(const Geometry& G, const Opnd<T>& L, const Opnd<T>& R, int n,
                                       uint32_t i) {
    const int kmin = imax(imax(R.lo, 0), n - L.hi);
    const int kmax = imin(imin(R.hi, n), n - L.lo);
    T acc = T(0);
    if (kmin > kmax) return acc;
    uint32_t q = i, r = 0, p = 1;
    for (int k = 0; k < kmin; ++k) {
        uint32_t qq, rr;
        G.divw.divmod(q, qq, rr);
        r += rr * p;
        p *= static_cast<uint32_t>(G.width);
        q = qq;
    }
    if constexpr (Pipelined) {
        T lv = L.p[G.db[n - kmin] + q], rv = R.p[G.db[kmin] + r];
        for (int k = kmin; k < kmax; ++k) {
            uint32_t qq, rr;
            G.divw.divmod(q, qq, rr);
            r += rr * p;
            p *= static_cast<uint32_t>(G.width);
            q = qq;
            const T ln = L.p[G.db[n - k - 1] + q], rn = R.p[G.db[k + 1] + r];
            acc = fma(lv, rv, acc);
            lv = ln;
            rv = rn;
        }
        return fma(lv, rv, acc);
    } else {
        for (int k = kmin;; ++k) {
            acc = fma(L.p[G.db[n - k] + q], R.p[G.db[k] + r], acc);
            if (k == kmax) break;
            uint32_t qq, rr;
            G.divw.divmod(q, qq, rr);
            r += rr * p;
            p *= static_cast<uint32_t>(G.width);
            q = qq;
        }
        return acc;
    }
}

// Copy levels [lo, hi] of a tensor into the same positions of a shared buffer.
template <typename T>
__device__ __forceinline__ void stage(T* dst, const T* src, int lo, int hi, const Geometry& G) {
    if (lo > hi) return;
    const uint32_t b = G.db[lo], e = G.db[hi + 1];
    for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) dst[i] = src[i];
}

// out[n] = alpha*add[n] + beta * L (x) R at level n, for n in [lo, hi], top
// degree first; `sync` puts a barrier after each degree (needed when L or R
// alias the destination in global memory).  Scale = false drops the multiply
// by beta (beta = 1) at compile time: a run-time test of beta == 1 in this
// loop measured 13 % slower on the Lie-increment step than the multiply.
template <typename T, bool Scale = true, bool Pipelined = false>
__device__ void product_levels(const Geometry& G, T* dst, int lo, int hi, const Opnd<T>& add,
                               T alpha, const Opnd<T>& L, const Opnd<T>& R, T beta, bool sync) {
    for (int n = hi; n >= lo; --n) {
        const uint32_t size = G.pw[n];
        const uint32_t base = G.db[n];
        const bool has_add = add.p != nullptr && add.lo <= n && n <= add.hi;
        for (uint32_t i = threadIdx.x; i < size; i += blockDim.x) {
            const T av = has_add ? add.p[base + i] : T(0);  // issued before the sum's loads
            T val = split_sum<Pipelined>(G, L, R, n, i);
            if constexpr (Scale) val *= beta;
            if (has_add) val = fma(alpha, av, val);
            dst[base + i] = val;
        }
        if (sync) __syncthreads();
    }
}

// One Horner intermediate on work buffer `o` (shared or global), following
// include/rpp/gpu/block/operations/intermediate/ft_exp.hpp:66-81,
// ft_fmexp.hpp:61-83 and ft_log.hpp:66-83.  Every in-place product reads only
// lower degrees of `o` (the exponent/argument is truncated to degree >= 1), so
// a barrier per degree, top degree first, keeps it exact.
//
// exp and fmexp run the Horner recursion o_d = A + (o_{d+1} (x) X) / d
// (A = 1 or M, d = D..1, o_{D+1} = A) rescaled: with p_d = c_d o_d and
// c_d = D!/(d-1)!,
//     p_d = c_d A + p_{d+1} (x) X,      o_1 = p_1 / D!,
// the same values up to rounding, with no multiply by 1/d on every output of
// every round -- one scaling pass at the end instead.  Depths above
// kScaledHornerMaxDepth keep the per-round scaling, so that the scaled values
// (up to D! times the result) stay far from FP32 overflow.
constexpr int kScaledHornerMaxDepth = 12;

// 1/d and d as T (0 < d <= kMaxDepth + 1) and 1/d! (d <= kScaledHornerMaxDepth),
// each rounded once at compile time: the values a run-time division gives (it
// is correctly rounded; d! is exact in both types up to 12!), without the
// FP64 instruction sequence a division costs every thread of the CTA on every
// Horner round.
template <typename T>
struct Reciprocals {
    T inv[kMaxDepth + 2];
    T num[kMaxDepth + 2];
    T inv_fact[kScaledHornerMaxDepth + 1];
    constexpr Reciprocals() : inv{}, num{}, inv_fact{} {
        for (int d = 1; d < kMaxDepth + 2; ++d) {
            inv[d] = T(1) / T(d);
            num[d] = T(d);
        }
        T f = T(1);
        inv_fact[0] = T(1);
        for (int d = 1; d <= kScaledHornerMaxDepth; ++d) {
            f *= T(d);
            inv_fact[d] = T(1) / f;
        }
    }
};
static __constant__ Reciprocals<double> kRecip64{};
static __constant__ Reciprocals<float> kRecip32{};
template <typename T>
__device__ __forceinline__ const Reciprocals<T>& recip();
template <>
__device__ __forceinline__ const Reciprocals<double>& recip<double>() {
    return kRecip64;
}
template <>
__device__ __forceinline__ const Reciprocals<float>& recip<float>() {
    return kRecip32;
}

template <typename T>
__device__ void intermediate_one(const Geometry& G, IntermediateKind kind, T* o, int olo, int ohi,
                                 Opnd<T> X, Opnd<T> M) {
    const int D = G.depth;
    // initialisation: set_identity / assign / set_constant
    if (olo <= ohi) {
        const uint32_t bgn = G.db[olo], end = G.db[ohi + 1];
        for (uint32_t i = bgn + threadIdx.x; i < end; i += blockDim.x) {
            T v = T(0);
            if (kind == IntermediateKind::FMExp) {
                const uint32_t mb = M.lo <= M.hi ? G.db[M.lo] : 0, me = M.lo <= M.hi ? G.db[M.hi + 1] : 0;
                if (i >= mb && i < me) v = M.p[i];
            }
            o[i] = v;
        }
    }
    __syncthreads();
    if (kind == IntermediateKind::Exp && threadIdx.x == 0 && olo == 0) o[0] = T(1);
    __syncthreads();
    const Opnd<T> none{nullptr, 1, 0};
    const bool scaled = kind != IntermediateKind::Log && D <= kScaledHornerMaxDepth;
    T c = T(1);  // c_{d+1}, then c_d after the update below
    for (int d = D; d > 0; --d) {
        const int tmax = D - d + 1;
        const Opnd<T> Xt{X.p, imax(1, X.lo), imin(X.hi, tmax)};
        const T inv = recip<T>().inv[d];
        c *= recip<T>().num[d];
        if (kind == IntermediateKind::Exp) {
            if (scaled) product_levels<T, false, true>(G, o, olo, ohi, none, T(0), Opnd<T>{o, olo, ohi}, Xt, T(1), true);
            else product_levels<T, true, true>(G, o, olo, ohi, none, T(0), Opnd<T>{o, olo, ohi}, Xt, inv, true);
            if (threadIdx.x == 0 && olo == 0) o[0] += scaled ? c : T(1);
            __syncthreads();
        } else if (kind == IntermediateKind::FMExp) {
            if (scaled) product_levels<T, false, true>(G, o, olo, ohi, M, c, Opnd<T>{o, olo, ohi}, Xt, T(1), true);
            else product_levels<T, true, true>(G, o, olo, ohi, M, T(1), Opnd<T>{o, olo, ohi}, Xt, inv, true);
        } else {
            if (threadIdx.x == 0 && olo == 0) o[0] += (d % 2 == 0) ? -inv : inv;  // (-1)^{d+1} / d
            __syncthreads();
            const int thi = imin(ohi, tmax);
            product_levels<T, false, true>(G, o, olo, thi, none, T(0), Opnd<T>{o, olo, thi}, Xt, T(1), true);
        }
    }
    if (scaled && olo <= ohi) {  // o = p_1 / D!
        const T s = recip<T>().inv_fact[D];  // 1 / c, c = D! exactly
        for (uint32_t i = G.db[olo] + threadIdx.x; i < G.db[ohi + 1]; i += blockDim.x) o[i] *= s;
        __syncthreads();
    }
}

}  // namespace ftdev
}  // namespace rpp_gb
