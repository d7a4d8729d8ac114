// ft_ops.cu -- per-operation sm_103a kernels of the batched free-tensor path:
// products (ft_mul, ft_fma, the in-place FMAs, ft_inplace_mul), the Horner
// intermediates (ft_exp, ft_fmexp, ft_log), the adjoint multiplies, the
// generalised antipode and the assign/identity helpers.
//
// Shape: one CTA per batch element (grid-stride over the batch).  When the
// operands fit, their in-range levels are staged in shared memory so every
// split of the product reads on-chip memory; otherwise the kernels read
// global memory directly and keep in-place updates correct by writing output
// degrees from the top down with a CTA barrier per degree (the order the
// reference's in-place kernels use, include/rpp/gpu/block/operations/basic/
// ft_inplace_fma.hpp:48-92).
//
// Products: out[n][i] = beta * sum_k L[n-k][i / W^k] * R[k][i % W^k] with the
// split degree k restricted to both operands' degree ranges (zero extension,
// include/rpp/gpu/block/operations/basic/detail/ft_multiply.hpp:14-64).  The
// splits are walked with one divide-by-W per step (FastDiv), no per-element
// degree search.
#include <cstdio>
#include <type_traits>

#include "bulk_stage.cuh"
#include "common.cuh"
#include "ft_device.cuh"
#include "launch_util.cuh"
#include "ops.hpp"

namespace rpp_gb {
namespace {

using namespace ftdev;

// Scale = false: beta is 1 and the products are not multiplied by it (one
// FP64 multiply per output coefficient saved; chosen by the launcher).
template <typename T, bool Scale>
__global__ void __launch_bounds__(256) k_product(Geometry G, ProductKind kind, TArg<T> out,
                                                 TArg<T> x, TArg<T> y, TArg<T> z, int64_t batch,
                                                 T alpha, T beta, int staged) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* sm = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    const uint32_t pd = staged_elems<T>(G.dim);
    uint32_t phase = 0;
    if (staged) bulk_stage_init(bar);
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        T* dst = out.at(b);
        // The three operand slots, in global memory.
        Opnd<T> add{nullptr, 1, 0}, L{nullptr, 1, 0}, R{nullptr, 1, 0};
        Opnd<T> self{dst, out.lo, out.hi};
        switch (kind) {
            case ProductKind::Fma:
                if (x.p) add = {x.at(b), x.lo, x.hi};
                L = {y.at(b), y.lo, y.hi};
                R = {z.at(b), z.lo, z.hi};
                break;
            case ProductKind::InplaceBCA:
                add = self;
                L = {y.at(b), y.lo, y.hi};
                R = {z.at(b), z.lo, z.hi};
                break;
            case ProductKind::InplaceABC:
                add = {z.at(b), z.lo, z.hi};
                L = self;
                R = {y.at(b), y.lo, y.hi};
                break;
            case ProductKind::InplaceBAC:
                add = {z.at(b), z.lo, z.hi};
                L = {y.at(b), y.lo, y.hi};
                R = self;
                break;
            case ProductKind::InplaceMul:
                L = self;
                R = {y.at(b), y.lo, y.hi};
                break;
        }
        if (staged) {
            // Snapshot every operand that is read (old values of an in-place
            // destination included) so the outputs can be written in any order.
            BulkStage<T> st(bar, phase);
            if (add.p) add.p = st.add(sm, add.p, add.lo, imin(add.hi, G.depth), G);
            L.p = st.add(sm + pd, L.p, L.lo, imin(L.hi, G.depth), G);
            R.p = st.add(sm + 2 * pd, R.p, R.lo, imin(R.hi, G.depth), G);
            if (!st.commit(G.fault)) return;
            product_levels<T, Scale>(G, dst, out.lo, imin(out.hi, G.depth), add, alpha, L, R, beta, false);
            bulk_stage_reuse();
        } else {
            product_levels<T, Scale>(G, dst, out.lo, imin(out.hi, G.depth), add, alpha, L, R, beta, true);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_intermediate(Geometry G, IntermediateKind kind, TArg<T> out,
                                                      TArg<T> x, TArg<T> m, int64_t batch,
                                                      int staged) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* sm = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    const uint32_t pd = staged_elems<T>(G.dim);
    uint32_t phase = 0;
    if (staged) bulk_stage_init(bar);
    const int ohi = imin(out.hi, G.depth);
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        Opnd<T> X{x.at(b), imax(1, x.lo), imin(x.hi, G.depth)};
        Opnd<T> M{nullptr, 1, 0};
        if (kind == IntermediateKind::FMExp) M = {m.at(b), m.lo, imin(m.hi, G.depth)};
        T* o = out.at(b);
        if (staged) {
            T* s_o = sm;
            BulkStage<T> st(bar, phase);
            X.p = st.add(sm + pd, X.p, X.lo, X.hi, G);
            if (M.p) M.p = st.add(sm + 2 * pd, M.p, M.lo, M.hi, G);
            if (!st.commit(G.fault)) return;
            intermediate_one(G, kind, s_o, out.lo, ohi, X, M);
            __syncthreads();
            if (out.lo <= ohi)
                for (uint32_t i = G.db[out.lo] + threadIdx.x; i < G.db[ohi + 1]; i += blockDim.x) o[i] = s_o[i];
            bulk_stage_reuse();
        } else {
            intermediate_one(G, kind, o, out.lo, ohi, X, M);
            __syncthreads();
        }
    }
}

// Adjoint multiplies (include/rpp/operations/basic/ft_adj_lmul.hpp,
// ft_adj_rmul.hpp; semantics as tests/rpp/ft_adjoint_test_helper.hpp:55-87):
//   left:  out[m][j] = sum_p sum_u op[p][u] arg[m+p][u*W^m + j]
//   right: out[m][j] = sum_p sum_v op[p][v] arg[m+p][j*W^p + v]
// The terms (p, u) of one coefficient form one run (a thread's offset is
// carried from split degree to split degree, so short splits do not leave
// lanes idle).  Output degrees with at least one coefficient per thread give
// each coefficient a thread.  Narrower degrees give each coefficient a group
// of g threads that stride over its terms and are then summed in a fixed
// order:
//  * right: g (a power of two) consecutive threads per coefficient, so their
//    reads arg[m+p][j*W^p + u] are consecutive; summed by an xor-shuffle
//    tree inside the warp, then (g > 32) the group's warps in warp order;
//  * left: threads t = j + r*W^m, so consecutive threads read consecutive
//    arg[m+p][u*W^m + j] (one thread per u would put the lanes of a warp
//    W^m elements apart, in few banks); lanes of a warp with the same j are
//    summed by a shuffle tree, then the warps' partials in warp order.
// The degree-0 coefficient of W16 D3 alone has 4 369 terms; W2 D12 has
// about 8 000 terms per output degree, most of them in the narrow degrees.
template <typename T>
__global__ void __launch_bounds__(256) k_adjoint(Geometry G, int left, TArg<T> out, TArg<T> op,
                                                 TArg<T> arg, int64_t batch, int staged) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* sm = reinterpret_cast<T*>(smem_raw + kBulkHeader);
    const uint32_t pd = staged_elems<T>(G.dim);
    // staged: 0 = nothing, 1 = both operands, 2 = the op only (arg read
    // through L1/L2 -- in both mappings a warp's lanes read consecutive
    // argument coefficients)
    T* s_part = sm + (staged == 1 ? 2 * pd : staged == 2 ? pd : 0);  // one partial per thread
    uint32_t phase = 0;
    if (staged) bulk_stage_init(bar);
    const int D = G.depth;
    const int ohi = imin(out.hi, D), phi = imin(op.hi, D), ahi = imin(arg.hi, D);
    const uint32_t nt = blockDim.x, t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const T* P = op.at(b);
        const T* A = arg.at(b);
        T* o = out.at(b);
        if (staged) {
            BulkStage<T> st(bar, phase);
            P = st.add(sm, P, op.lo, phi, G);
            if (staged == 1) A = st.add(sm + pd, A, arg.lo, ahi, G);
            if (!st.commit(G.fault)) return;
        }
        for (int m = out.lo; m <= ohi; ++m) {
            const uint32_t wm = G.pw[m];
            const int pmin = imax(op.lo, arg.lo - m), pmax = imin(phi, ahi - m);
            // terms u = first, first + stride, ... of coefficient j, over the
            // split degrees in turn
            auto terms = [&](uint32_t j, uint32_t first, uint32_t stride) {
                T acc = T(0);
                uint32_t u = first;
                for (int p = pmin; p <= pmax; ++p) {
                    const uint32_t wp = G.pw[p];
                    const T* Pp = P + G.db[p];
                    const T* Ap = A + G.db[m + p];
                    if (left)
                        for (; u < wp; u += stride) acc = fma(Pp[u], Ap[u * wm + j], acc);
                    else
                        for (; u < wp; u += stride) acc = fma(Pp[u], Ap[j * wp + u], acc);
                    u -= wp;
                }
                return acc;
            };
            if (wm >= nt) {
                for (uint32_t j = t; j < wm; j += nt) o[G.db[m] + j] = terms(j, 0, 1);
            } else if (!left) {
                uint32_t g = 1;
                while (2 * g * wm <= nt) g *= 2;
                const uint32_t j = t / g, r = t % g;
                T acc = j < wm ? terms(j, r, g) : T(0);
                for (uint32_t off = (g < 32 ? g : 32) / 2; off > 0; off /= 2) acc += __shfl_xor_sync(0xffffffffu, acc, off);
                if (g <= 32) {
                    if (j < wm && r == 0) o[G.db[m] + j] = acc;
                } else {
                    if (lane == 0) s_part[warp] = acc;
                    __syncthreads();
                    const uint32_t gw = g / 32;
                    if (j < wm && r == 0) {
                        T v = s_part[warp];
                        for (uint32_t k = 1; k < gw; ++k) v += s_part[warp + k];
                        o[G.db[m] + j] = v;
                    }
                    __syncthreads();
                }
            } else {
                const uint32_t g = nt / wm;
                const uint32_t j = t % wm, r = t / wm;
                T acc = r < g ? terms(j, r, g) : T(0);
                if (wm < 32) {
                    // lanes l, l + wm, l + 2wm, ... of a warp share j
                    for (uint32_t off = wm; off < 32u; off *= 2u) {
                        const T x = __shfl_down_sync(0xffffffffu, acc, off);
                        if (lane + off < 32u) acc += x;
                    }
                    if (lane < wm) s_part[warp * wm + t % wm] = acc;
                } else {
                    s_part[t] = acc;
                }
                __syncthreads();
                if (t < wm) {
                    T v = T(0);
                    if (wm < 32)
                        for (uint32_t w = 0; w < (nt >> 5); ++w) v += s_part[w * wm + t];
                    else
                        for (uint32_t k = 0; k < g; ++k) v += s_part[t + k * wm];
                    o[G.db[m] + t] = v;
                }
                __syncthreads();
            }
        }
        bulk_stage_reuse();
    }
}

__device__ __forceinline__ int level_of(const Geometry& G, uint32_t idx) {
    int n = 0;
    while (n < G.depth && G.db[n + 1] <= idx) ++n;
    return n;
}

// Generalised antipode (include/rpp/gpu/block/operations/basic/
// tensor_generalised_antipode.hpp:44-75): out[rev w] = sign(|w|) arg[w] on
// out's degree range; degrees missing from arg are zeroed.
template <typename T>
__global__ void k_antipode(Geometry G, int sign, TArg<T> out, TArg<T> arg, int64_t batch) {
    const int ohi = imin(out.hi, G.depth);
    if (out.lo > ohi) return;
    const uint32_t bgn = G.db[out.lo], end = G.db[ohi + 1];
    for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
        const T* A = arg.at(b);
        T* o = out.at(b);
        for (uint32_t idx = bgn + blockIdx.x * blockDim.x + threadIdx.x; idx < end;
             idx += gridDim.x * blockDim.x) {
            const int n = level_of(G, idx);
            const uint32_t i = idx - G.db[n];
            if (arg.lo <= n && n <= arg.hi) {
                uint32_t rev = 0, t = i;
                for (int d = 0; d < n; ++d) {
                    uint32_t q, r;
                    G.divw.divmod(t, q, r);
                    rev = rev * static_cast<uint32_t>(G.width) + r;
                    t = q;
                }
                const T v = A[idx];
                o[G.db[n] + rev] = (sign && (n & 1)) ? -v : v;
            } else {
                o[idx] = T(0);
            }
        }
    }
}

// vector_assign / vector_set_constant / tensor_set_identity /
// tensor_add_identity (include/rpp/gpu/block/operations/linalg/
// vector_assign.hpp:51-112, vector_set_constant.hpp:42-78,
// basic/tensor_set_identity.hpp:48-57, basic/tensor_add_identity.hpp:37-45).
template <typename T>
__global__ void k_helper(Geometry G, HelperKind kind, TArg<T> out, TArg<T> arg, int64_t batch, T value) {
    const int ohi = imin(out.hi, G.depth);
    for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
        T* o = out.at(b);
        if (kind == HelperKind::AddIdentity) {
            if (blockIdx.x == 0 && threadIdx.x == 0 && out.lo == 0) o[0] = o[0] + value;
            continue;
        }
        if (out.lo > ohi) continue;
        const uint32_t bgn = G.db[out.lo], end = G.db[ohi + 1];
        uint32_t cb = 0, ce = 0;
        const T* A = nullptr;
        if (kind == HelperKind::Assign) {
            const int lo = imax(out.lo, arg.lo), hi = imin(ohi, imin(arg.hi, G.depth));
            if (lo <= hi) {
                cb = G.db[lo];
                ce = G.db[hi + 1];
            }
            A = arg.at(b);
        }
        for (uint32_t idx = bgn + blockIdx.x * blockDim.x + threadIdx.x; idx < end;
             idx += gridDim.x * blockDim.x) {
            T v = kind == HelperKind::SetConstant ? value : T(0);
            if (kind == HelperKind::Assign && idx >= cb && idx < ce) v = A[idx];
            if (kind == HelperKind::SetIdentity && idx == 0) v = value;
            o[idx] = v;
        }
    }
}

// Vector-Jacobian product of the exponential of a degree-one tensor (the
// last step of the stored-prefix reverse pass composed from the reference's
// operations): given x (W letters) and a cotangent H of E = exp(x), writes
//     dx_a = sum_w H[w] dE[w]/dx_a.
// E_n = E_{n-1} (x) x / n for a degree-one x, so the reverse of that Horner
// recursion is, top level first,
//     Ebar_{n-1}[u] += sum_a Ebar_n[ua] x_a / n,   dx_a += sum_u Ebar_n[ua] E_{n-1}[u] / n,
// with Ebar = H initially.  One CTA per batch element; E and Ebar below the
// top level in shared memory (2 * db[D] elements: the recursion never reads
// E_D, and Ebar_D = H_D is only read, straight from global memory -- so the
// widest states fit, 149 KB at W6 D6 FP64), one partial sum per thread for dx.
template <typename T>
__global__ void __launch_bounds__(256) k_exp_letter_vjp(Geometry G, const T* H, int64_t h_stride, const T* x,
                                                        int64_t x_stride, T* dx, int64_t dx_stride,
                                                        int64_t batch) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int D = G.depth;
    const uint32_t lo = G.db[D];  // coefficients below the top level
    T* E = reinterpret_cast<T*>(smem_raw);
    T* Eb = E + lo;
    T* part = Eb + lo;
    const uint32_t W = static_cast<uint32_t>(G.width);
    const uint32_t slots = blockDim.x / W;
    const uint32_t my_a = threadIdx.x % W, my_slot = threadIdx.x / W;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const T* xb = x + b * x_stride;
        const T* hb = H + b * h_stride;
        for (uint32_t i = threadIdx.x; i < lo; i += blockDim.x) Eb[i] = hb[i];
        if (threadIdx.x == 0) E[0] = T(1);
        __syncthreads();
        for (int n = 1; n < D; ++n) {
            const T inv = recip<T>().inv[n];
            for (uint32_t i = threadIdx.x; i < G.pw[n]; i += blockDim.x) {
                uint32_t q, a;
                G.divw.divmod(i, q, a);
                E[G.db[n] + i] = E[G.db[n - 1] + q] * (xb[a] * inv);
            }
            __syncthreads();
        }
        T acc = T(0);
        for (int n = D; n >= 1; --n) {
            const T inv = recip<T>().inv[n];
            const uint32_t wp = G.pw[n - 1];
            const T* En1 = E + G.db[n - 1];
            const T* Ebn = n == D ? hb + lo : Eb + G.db[n];
            T* Ebn1 = Eb + G.db[n - 1];
            for (uint32_t u = threadIdx.x; u < wp; u += blockDim.x) {
                T s = T(0);
                for (uint32_t a = 0; a < W; ++a) s = fma(Ebn[u * W + a], xb[a], s);
                Ebn1[u] = fma(s, inv, Ebn1[u]);
            }
            if (my_slot < slots)
                for (uint32_t u = my_slot; u < wp; u += slots) acc = fma(Ebn[u * W + my_a], En1[u] * inv, acc);
            __syncthreads();
        }
        part[threadIdx.x] = my_slot < slots ? acc : T(0);
        __syncthreads();
        if (threadIdx.x < W) {
            T v = T(0);
            for (uint32_t s2 = 0; s2 < slots; ++s2) v += part[s2 * W + threadIdx.x];
            dx[b * dx_stride + threadIdx.x] = v;
        }
        __syncthreads();
    }
}

constexpr size_t kStageLimit = 200 * 1024;

}  // namespace

template <typename T>
cudaError_t launch_product(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, ProductKind kind,
                           TArg<T> out, TArg<T> x, TArg<T> y, TArg<T> z, int64_t batch, double alpha,
                           double beta) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem_need = kBulkHeader + 3 * static_cast<size_t>(staged_elems<T>(g.dim)) * sizeof(T);
    const int staged = smem_need <= kStageLimit && smem_need <= static_cast<size_t>(dev.max_smem_optin);
    const size_t smem = staged ? smem_need : 0;
    const int threads = threads_for(g.pw[g.depth]);
    auto run = [&](auto kernel) {
        cudaError_t err = allow_large_smem<decltype(kernel)::value>(dev);
        if (err != cudaSuccess) return err;
        dim3 grid;
        if ((err = batch_grid(decltype(kernel)::value, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
        decltype(kernel)::value<<<grid, threads, smem, s>>>(g, kind, out, x, y, z, batch, static_cast<T>(alpha),
                                                            static_cast<T>(beta), staged);
        return cudaGetLastError();
    };
    if (static_cast<T>(beta) == T(1)) return run(std::integral_constant<decltype(&k_product<T, false>), &k_product<T, false>>{});
    return run(std::integral_constant<decltype(&k_product<T, true>), &k_product<T, true>>{});
}

template <typename T>
cudaError_t launch_intermediate(const Geometry& g, const DeviceInfo& dev, cudaStream_t s,
                                IntermediateKind kind, TArg<T> out, TArg<T> x, TArg<T> m,
                                int64_t batch) {
    if (batch <= 0) return cudaSuccess;
    constexpr auto kernel = k_intermediate<T>;
    cudaError_t err = allow_large_smem<kernel>(dev);
    if (err != cudaSuccess) return err;
    const size_t smem_need =
        kBulkHeader + (kind == IntermediateKind::FMExp ? 3 : 2) * static_cast<size_t>(staged_elems<T>(g.dim)) * sizeof(T);
    const int staged = smem_need <= kStageLimit && smem_need <= static_cast<size_t>(dev.max_smem_optin);
    const size_t smem = staged ? smem_need : 0;
    const int threads = threads_for(g.pw[g.depth]);
    dim3 grid;
    if ((err = batch_grid(kernel, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
    kernel<<<grid, threads, smem, s>>>(g, kind, out, x, m, batch, staged);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adjoint(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, bool left,
                           TArg<T> out, TArg<T> op, TArg<T> arg, int64_t batch) {
    if (batch <= 0) return cudaSuccess;
    constexpr auto kernel = k_adjoint<T>;
    cudaError_t err = allow_large_smem<kernel>(dev);
    if (err != cudaSuccess) return err;
    // Both operands staged while that leaves two or more CTAs per SM; when it
    // would leave one (W2 D12 FP64: 131 KB), the op alone, for three CTAs per
    // SM (W2 D12, batch 16 384: ft_adj_lmul 4.46 -> 3.90 ms, ft_adj_rmul 4.56 ->
    // 4.15 ms; at W16 D3, 70 KB for both and three CTAs per SM, op-only staging
    // measured slower).
    const size_t one = static_cast<size_t>(staged_elems<T>(g.dim)) * sizeof(T);
    const size_t part = kBulkHeader + 256 * sizeof(T);  // the mbarrier and one partial per thread
    const size_t limit = std::min(kStageLimit, static_cast<size_t>(dev.max_smem_optin));
    int per_sm = 0;
    if ((err = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev.device)) != cudaSuccess)
        return err;
    int staged = 0;
    if (2 * one + part <= limit && 2 * (2 * one + part + 1024) <= static_cast<size_t>(per_sm))
        staged = 1;
    else if (one + part <= limit)
        staged = 2;
    const size_t smem = (staged == 1 ? 2 * one : staged == 2 ? one : 0) + part;
    const int threads = threads_for(g.pw[g.depth]);
    dim3 grid;
    if ((err = batch_grid(kernel, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
    kernel<<<grid, threads, smem, s>>>(g, left ? 1 : 0, out, op, arg, batch, staged);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_antipode(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, bool sign,
                            TArg<T> out, TArg<T> arg, int64_t batch) {
    if (batch <= 0) return cudaSuccess;
    const int threads = 256;
    const uint32_t span = g.dim;
    const unsigned gx = (span + threads - 1) / threads;
    const unsigned gy = static_cast<unsigned>(std::min<int64_t>(batch, 65535));
    k_antipode<T><<<dim3(gx, gy), threads, 0, s>>>(g, sign ? 1 : 0, out, arg, batch);
    (void)dev;
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_helper(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, HelperKind kind,
                          TArg<T> out, TArg<T> arg, int64_t batch, double value) {
    if (batch <= 0) return cudaSuccess;
    const int threads = 256;
    const unsigned gx = (g.dim + threads - 1) / threads;
    const unsigned gy = static_cast<unsigned>(std::min<int64_t>(batch, 65535));
    k_helper<T><<<dim3(gx, gy), threads, 0, s>>>(g, kind, out, arg, batch, static_cast<T>(value));
    (void)dev;
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_exp_letter_vjp(const Geometry& g, const DeviceInfo& dev, cudaStream_t s, const T* H,
                                  int64_t h_stride, const T* x, int64_t x_stride, T* dx, int64_t dx_stride,
                                  int64_t batch) {
    if (batch <= 0) return cudaSuccess;
    constexpr auto kernel = k_exp_letter_vjp<T>;
    cudaError_t err = allow_large_smem<kernel>(dev);
    if (err != cudaSuccess) return err;
    const int threads = threads_for(g.pw[g.depth]);
    if (threads < g.width) return cudaErrorInvalidConfiguration;
    const size_t smem = (2 * static_cast<size_t>(g.db[g.depth]) + threads) * sizeof(T);
    if (smem > static_cast<size_t>(dev.max_smem_optin)) return cudaErrorInvalidConfiguration;
    dim3 grid;
    if ((err = batch_grid(kernel, dev, threads, smem, batch, grid)) != cudaSuccess) return err;
    kernel<<<grid, threads, smem, s>>>(g, H, h_stride, x, x_stride, dx, dx_stride, batch);
    return cudaGetLastError();
}

#define RPP_GB_INSTANTIATE(T)                                                                      \
    template cudaError_t launch_product<T>(const Geometry&, const DeviceInfo&, cudaStream_t,       \
                                           ProductKind, TArg<T>, TArg<T>, TArg<T>, TArg<T>,        \
                                           int64_t, double, double);                               \
    template cudaError_t launch_intermediate<T>(const Geometry&, const DeviceInfo&, cudaStream_t,  \
                                                IntermediateKind, TArg<T>, TArg<T>, TArg<T>,       \
                                                int64_t);                                          \
    template cudaError_t launch_adjoint<T>(const Geometry&, const DeviceInfo&, cudaStream_t, bool, \
                                           TArg<T>, TArg<T>, TArg<T>, int64_t);                    \
    template cudaError_t launch_antipode<T>(const Geometry&, const DeviceInfo&, cudaStream_t,      \
                                            bool, TArg<T>, TArg<T>, int64_t);                      \
    template cudaError_t launch_helper<T>(const Geometry&, const DeviceInfo&, cudaStream_t,        \
                                          HelperKind, TArg<T>, TArg<T>, int64_t, double);          \
    template cudaError_t launch_exp_letter_vjp<T>(const Geometry&, const DeviceInfo&, cudaStream_t, \
                                                  const T*, int64_t, const T*, int64_t, T*, int64_t,  \
                                                  int64_t);

RPP_GB_INSTANTIATE(float)
RPP_GB_INSTANTIATE(double)

}  // namespace rpp_gb
