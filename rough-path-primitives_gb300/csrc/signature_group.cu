// signature_group.cu -- several signature jobs (different (width, depth)
// and precisions) in one persistent launch: rpp_gb_signature_group.
#include "signature_letters.cuh"

namespace rpp_gb {

// ---------------------------------------------------------------------------
// Grouped launch (rpp_gb_signature_group).
//
// Several jobs -- batches of different (width, depth) and precision -- run in
// one persistent launch.  A CTA works through the jobs in the order the
// ordering kernel chose (the job whose most expensive path costs most first,
// so the cheapest paths of the last job fill the tail).  For job j it splits
// into teams[j] teams of team_threads[j] threads, each with its own slice of
// the dynamic shared memory and its own named barrier; every team takes paths
// of job j from the job's work counter (longest first for ragged batches)
// until none is left, then the CTA moves on to the next job.  A path is run
// by run_path with the team in place of a CTA, so its outputs equal those of
// a separate rpp_gb_signature call whose CTA size is the team size.
namespace {

// One job as the kernels see it.  The kernel parameters stay far below the
// 4 KB of a classic parameter block: the geometry is rebuilt on the device
// from (width, depth) and the host's divider.
struct GroupJob {
    int32_t width;
    int32_t depth;
    int32_t fp64;
    int32_t mode;
    int32_t letters;      // FP32: warp-per-letter teams (signature_letters.cuh), forward-only or forward + reverse
    int32_t cot;          // FP64 forward + reverse: cotangent arrays in the workspace gws
    uint32_t team_threads;
    uint32_t teams;
    uint32_t slice;       // shared-memory bytes of one team (a multiple of 16)
    uint32_t fd_m, fd_l;  // the host's FastDiv of the width
    uint32_t* fault;
    const void* incr;
    const int64_t* offsets;
    int64_t length;
    int64_t batch;
    int64_t weight;  // estimated cost of one increment for one team (ordering key)
    void* sig;
    int64_t sig_stride;
    const void* seed;
    int64_t seed_stride;
    void* grad;
    int32_t* order;         // ragged jobs: the paths longest first (scratch)
    unsigned int* counter;  // the job's work counter (scratch)
    void* gws;              // cot jobs: one slice of gws_stride elements per team of the launch
    int64_t gws_stride;
};

struct GroupTable {
    GroupJob job[kMaxGroupJobs];
    int32_t njobs;
    int32_t* seq;  // the order in which CTAs take the jobs (scratch)
};
static_assert(sizeof(GroupTable) < 4096, "grouped launch parameters must fit a classic parameter block");

// Job k of the table into `out`, with compile-time indices only (a run-time
// index into a parameter array would copy the table to local memory).
__device__ __forceinline__ void select_job(const GroupTable& tab, int j, GroupJob& out) {
#pragma unroll
    for (int k = 0; k < kMaxGroupJobs; ++k)
        if (k == j) out = tab.job[k];
}

// The geometry of plan (width, depth) as rpp_gb_plan_create builds it, plus
// the chain offsets of make_sig_geometry.
__device__ void build_sig_geometry(const GroupJob& job, SigGeometry& sg) {
    Geometry& g = sg.g;
    g.width = job.width;
    g.depth = job.depth;
    uint32_t db = 0, pw = 1;
    for (int n = 0; n <= job.depth; ++n) {
        g.db[n] = db;
        g.pw[n] = pw;
        db += pw;
        pw *= static_cast<uint32_t>(job.width);
    }
    g.db[job.depth + 1] = db;
    g.pw[job.depth + 1] = 0;
    g.dim = db;
    g.divw.d = static_cast<uint32_t>(job.width);
    g.divw.m = job.fd_m;
    g.divw.l = job.fd_l;
    g.fault = job.fault;
    uint32_t acc = 0;
    for (int j = 0; j <= job.depth; ++j) {
        sg.choff[j] = acc;
        if (j < job.depth) acc += static_cast<uint32_t>(job.depth - j) * g.pw[j];
    }
    sg.chain_total = acc;
}

// One CTA: the ragged jobs' paths longest first (a counting sort per job, as
// k_order_by_length), every job's counter zeroed, and the job sequence by
// decreasing cost of the job's most expensive path.
__global__ void __launch_bounds__(1024) k_order_group(GroupTable tab) {
    __shared__ unsigned int hist[kLengthBuckets];
    __shared__ unsigned int start[kLengthBuckets];
    __shared__ unsigned long long top[kMaxGroupJobs];
#pragma unroll
    for (int j = 0; j < kMaxGroupJobs; ++j) {
        if (j >= tab.njobs) break;
        const GroupJob& job = tab.job[j];
        if (threadIdx.x == 0) {
            top[j] = 0;
            *job.counter = 0;
        }
        if (!job.order) {
            if (threadIdx.x == 0) top[j] = static_cast<unsigned long long>(job.length) * job.weight;
            continue;
        }
        for (int i = threadIdx.x; i < kLengthBuckets; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        for (int64_t b = threadIdx.x; b < job.batch; b += blockDim.x) {
            const int64_t len = job.offsets[b + 1] - job.offsets[b];
            atomicAdd(&hist[length_bucket(len)], 1u);
            atomicMax(&top[j], static_cast<unsigned long long>(len) * job.weight);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int acc = 0;
            for (int k = kLengthBuckets - 1; k >= 0; --k) {
                start[k] = acc;
                acc += hist[k];
            }
        }
        __syncthreads();
        for (int64_t b = threadIdx.x; b < job.batch; b += blockDim.x) {
            const unsigned int pos = atomicAdd(&start[length_bucket(job.offsets[b + 1] - job.offsets[b])], 1u);
            job.order[pos] = static_cast<int32_t>(b);
        }
        __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int seq[kMaxGroupJobs];
        for (int j = 0; j < tab.njobs; ++j) {
            int k = j;
            while (k > 0 && top[seq[k - 1]] < top[j]) {
                seq[k] = seq[k - 1];
                --k;
            }
            seq[k] = j;
        }
        for (int j = 0; j < tab.njobs; ++j) tab.seq[j] = seq[j];
    }
}

// The grouped kernel's shared state, at file scope so that the team bodies
// (separate functions) address it as shared memory: the job in progress, its
// geometry, each team's broadcast slot, and the dynamic slices.
__shared__ SigGeometry g_sg;
__shared__ GroupJob g_job;
__shared__ int64_t g_task[15];
extern __shared__ __align__(16) unsigned char g_group_smem[];

// 640 threads at most: the team bodies then have 96 registers (at 64 -- 1024
// threads -- and 80 -- 768 threads -- their calls spilled).
constexpr int kGroupMaxThreads = 640;
constexpr int kGroupMaxTeams = 15;  // named barriers 1..15

// Team k's share of the current job: paths from the job's counter until none
// is left.  Not inlined: each (precision, width) body gets its own register
// allocation (inlined into one kernel, the sixteen bodies spilled).
// COT: the job keeps its cotangent level and chains in team slot
// blockIdx.x * teams + k of the workspace (kCotGlobal).
template <typename T, int WT, bool COT = false>
__device__ __noinline__ void group_team(const SubTeam tm, const uint32_t k) {
    const GroupJob& job = g_job;
    bool vec4 = false;
    SigShared<T> sh = place_arrays<T, WT, COT>(tm, g_sg, job.mode, COT ? static_cast<T*>(job.gws) : nullptr,
                                               job.gws_stride, g_group_smem + static_cast<size_t>(k) * job.slice,
                                               vec4, static_cast<int64_t>(blockIdx.x) * job.teams + k);
    for (;;) {
        if (tm.rank() == 0) g_task[k] = static_cast<int64_t>(atomicAdd(job.counter, 1u));
        tm.sync();
        const int64_t idx = g_task[k];
        if (idx >= job.batch) break;
        // (the slot is rewritten only after run_path's closing barrier)
        const int64_t b = job.order ? job.order[idx] : idx;
        const int64_t off = job.offsets ? job.offsets[b] : b * job.length;
        const int64_t len = job.offsets ? job.offsets[b + 1] - off : job.length;
        run_path<T, WT>(tm, g_sg, sh, static_cast<const T*>(job.incr), b, off, len, static_cast<T*>(job.sig),
                        job.sig_stride, static_cast<const T*>(job.seed), job.seed_stride, static_cast<T*>(job.grad),
                        job.mode, vec4);
    }
}

// Team k of W warps, one per first letter, on FP32 forward-only paths of the
// current job (the kernel of signature_fp32.cu, inside the group): each warp
// works through its slice of the path with __syncwarp only; the team meets on
// its named barrier to take the next path.
template <int W, int D>
__device__ __noinline__ void group_letters(const SubTeam tm, const uint32_t k) {
    const GroupJob& job = g_job;
    const uint32_t c = tm.rank() / 32, lane = tm.rank() % 32;
    float* region = reinterpret_cast<float*>(g_group_smem + static_cast<size_t>(k) * job.slice) +
                    c * LetterLayout<W, D>::warp_floats;
    for (;;) {
        if (tm.rank() == 0) g_task[k] = static_cast<int64_t>(atomicAdd(job.counter, 1u));
        tm.sync();
        const int64_t idx = g_task[k];
        tm.sync();  // every warp has read the slot before the leader rewrites it
        if (idx >= job.batch) break;
        const int64_t b = job.order ? job.order[idx] : idx;
        const int64_t off = job.offsets ? job.offsets[b] : b * job.length;
        const int64_t len = job.offsets ? job.offsets[b + 1] - off : job.length;
        letter_path<W, D>(static_cast<const float*>(job.incr), b, off, len, static_cast<float*>(job.sig),
                          job.sig_stride, region, c, lane);
    }
}

// Team k of W warps on FP32 forward + reverse paths of the current job (the
// kernel k_signature_letters_rev, inside the group): the warps meet on the
// team's named barrier once per 8 reverse steps (the letter gradients) and
// to take the next path.
template <int W, int D>
__device__ __noinline__ void group_letters_rev(const SubTeam tm, const uint32_t k) {
    using Rev = LetterRevLayout<W, D>;
    const GroupJob& job = g_job;
    const uint32_t c = tm.rank() / 32, lane = tm.rank() % 32;
    float* base = reinterpret_cast<float*>(g_group_smem + static_cast<size_t>(k) * job.slice);
    float* region = base + c * Rev::warp_floats;
    float* pbuf = base + W * Rev::warp_floats;
    for (;;) {
        if (tm.rank() == 0) g_task[k] = static_cast<int64_t>(atomicAdd(job.counter, 1u));
        tm.sync();
        const int64_t idx = g_task[k];
        tm.sync();  // every warp has read the slot before the leader rewrites it
        if (idx >= job.batch) break;
        const int64_t b = job.order ? job.order[idx] : idx;
        const int64_t off = job.offsets ? job.offsets[b] : b * job.length;
        const int64_t len = job.offsets ? job.offsets[b + 1] - off : job.length;
        letter_fwd_bwd<W, D>(tm, static_cast<const float*>(job.incr), b, off, len, static_cast<float*>(job.sig),
                             job.sig_stride, static_cast<const float*>(job.seed), job.seed_stride,
                             static_cast<float*>(job.grad), job.mode & (kForward | kBackward | kTopLevel), region,
                             pbuf, c, lane);
        tm.sync();  // the last block's partials are read before the next path writes pbuf
    }
}

template <int W, int D>
__device__ __forceinline__ void group_letters_rev_if(const SubTeam tm, const uint32_t k) {
    if constexpr (D >= 3) group_letters_rev<W, D>(tm, k);
}

__device__ __forceinline__ void group_letters_shape(const SubTeam tm, const uint32_t k) {
    if (g_job.mode & kBackward) {
        switch (g_job.width * 100 + g_job.depth) {
#define RPP_GB_LETTER_CASE(w, d) \
    case w * 100 + d: group_letters_rev_if<w, d>(tm, k); break;
            RPP_GB_LETTER_SHAPES(RPP_GB_LETTER_CASE)
#undef RPP_GB_LETTER_CASE
            default: break;
        }
        return;
    }
    switch (g_job.width * 100 + g_job.depth) {
#define RPP_GB_LETTER_CASE(w, d) \
    case w * 100 + d: group_letters<w, d>(tm, k); break;
        RPP_GB_LETTER_SHAPES(RPP_GB_LETTER_CASE)
#undef RPP_GB_LETTER_CASE
        default: break;
    }
}

template <typename T>
__device__ __forceinline__ void group_team_width(const SubTeam tm, const uint32_t k) {
    if constexpr (std::is_same<T, float>::value) {
        if (g_job.letters) {
            group_letters_shape(tm, k);
            return;
        }
    }
    if constexpr (std::is_same<T, double>::value) {
        if (g_job.cot) {
            switch (g_job.width) {
                case 2: group_team<T, 2, true>(tm, k); break;
                case 3: group_team<T, 3, true>(tm, k); break;
                case 4: group_team<T, 4, true>(tm, k); break;
                case 5: group_team<T, 5, true>(tm, k); break;
                case 6: group_team<T, 6, true>(tm, k); break;
                case 8: group_team<T, 8, true>(tm, k); break;
                case 16: group_team<T, 16, true>(tm, k); break;
                default: group_team<T, 0, true>(tm, k); break;
            }
            return;
        }
    }
    switch (g_job.width) {
        case 2: group_team<T, 2>(tm, k); break;
        case 3: group_team<T, 3>(tm, k); break;
        case 4: group_team<T, 4>(tm, k); break;
        case 5: group_team<T, 5>(tm, k); break;
        case 6: group_team<T, 6>(tm, k); break;
        case 8: group_team<T, 8>(tm, k); break;
        case 16: group_team<T, 16>(tm, k); break;
        default: group_team<T, 0>(tm, k); break;
    }
}

__global__ void __launch_bounds__(kGroupMaxThreads, 1) k_signature_group(GroupTable tab) {
    for (int q = 0; q < tab.njobs; ++q) {
        if (threadIdx.x == 0) {
            select_job(tab, tab.seq[q], g_job);
            build_sig_geometry(g_job, g_sg);
        }
        __syncthreads();
        const uint32_t t = g_job.team_threads;
        const uint32_t k = threadIdx.x / t;
        if (k < g_job.teams) {
            const SubTeam tm{threadIdx.x - k * t, t, 1 + k};
            if (g_job.fp64)
                group_team_width<double>(tm, k);
            else
                group_team_width<float>(tm, k);
        }
        __syncthreads();  // the job, its geometry and the slices are rewritten for the next job
    }
}

// Shared memory of one warp-per-letter team (W warps' regions), 0 for a
// shape without an instantiation.
size_t letter_slice_bytes(int width, int depth) {
    switch (width * 100 + depth) {
#define RPP_GB_LETTER_CASE(w, d) \
    case w * 100 + d: return (static_cast<size_t>(w) * LetterLayout<w, d>::warp_floats * sizeof(float) + 15) / 16 * 16;
        RPP_GB_LETTER_SHAPES(RPP_GB_LETTER_CASE)
#undef RPP_GB_LETTER_CASE
        default: return 0;
    }
}

// The same for a forward + reverse team (the W warps' regions and the
// team's letter-partials buffer), 0 without a reverse instantiation.
template <int W, int D>
size_t letter_rev_slice_bytes_shape() {
    if constexpr (D >= 3) {
        using Rev = LetterRevLayout<W, D>;
        return ((static_cast<size_t>(W) * Rev::warp_floats + Rev::pbuf_floats) * sizeof(float) + 15) / 16 * 16;
    } else {
        return 0;
    }
}

size_t letter_rev_slice_bytes(int width, int depth) {
    switch (width * 100 + depth) {
#define RPP_GB_LETTER_CASE(w, d) \
    case w * 100 + d: return letter_rev_slice_bytes_shape<w, d>();
        RPP_GB_LETTER_SHAPES(RPP_GB_LETTER_CASE)
#undef RPP_GB_LETTER_CASE
        default: return 0;
    }
}

// One team's shared memory for `job` (mode may gain kTopGlobal when the top
// level must go to global memory to fit `budget`); 0 when it cannot fit.
// With kCotGlobal the cotangent arrays are not in shared memory.
template <typename T>
size_t group_slice(const SigGeometry& sg, int threads, int& mode, size_t budget) {
    const bool bwd = (mode & kBackward) && !(mode & kCotGlobal);
    size_t smem = sig_smem_bytes<T>(sg, threads, bwd, true, (mode & kTopGlobal) != 0);
    if (smem > budget && !(mode & kTopGlobal)) {
        mode |= kTopGlobal;
        smem = sig_smem_bytes<T>(sg, threads, bwd, true, true);
    }
    smem = (smem + 15) / 16 * 16;
    return smem <= budget ? smem : 0;
}

}  // namespace

cudaError_t launch_signature_group(const DeviceInfo& dev, cudaStream_t s, const SignatureJob* jobs, int njobs,
                                   int schedule, GroupRefusal* refusal) {
    *refusal = GroupRefusal::None;
    if (njobs < 1 || njobs > kMaxGroupJobs || schedule < 0) return cudaErrorInvalidValue;
    const int cta = (schedule & 1023) ? (schedule & 1023) : kGroupMaxThreads;
    if (cta % 32 != 0 || cta > kGroupMaxThreads) return cudaErrorInvalidConfiguration;
    constexpr auto kernel = k_signature_group;
    cudaFuncAttributes attr{};
    cudaError_t err = cudaFuncGetAttributes(&attr, kernel);
    if (err != cudaSuccess) return err;
    const size_t optin = static_cast<size_t>(dev.max_smem_optin) - attr.sharedSizeBytes;
    GroupTable tab{};
    tab.njobs = njobs;
    size_t budget = 0;
    int64_t ragged = 0, needed_ctas = 0;
    for (int j = 0; j < njobs; ++j) {
        const SignatureJob& in = jobs[j];
        GroupJob& job = tab.job[j];
        const int t = in.threads;
        if (t % 32 != 0 || t > cta || t < in.g.depth * in.g.width || t < 32) return cudaErrorInvalidConfiguration;
        const SigGeometry sg = make_sig_geometry(in.g);
        job.mode = kForward | (in.sig ? kTopLevel : 0) | (in.seed && in.grad ? kBackward : 0);
        if ((schedule & kScheduleMergedReverse) && (job.mode & kBackward)) job.mode |= kMergedReverse;
        job.cot = in.cot && in.fp64 && (job.mode & kBackward) && !in.letters ? 1 : 0;
        if (job.cot) job.mode |= kCotGlobal;
        int mode = job.mode;
        size_t slice = in.fp64 ? group_slice<double>(sg, t, mode, optin) : group_slice<float>(sg, t, mode, optin);
        if (slice && !in.letters && !(mode & kTopGlobal)) {
            // the top level in the signature and seed rows where that lets
            // more teams share a CTA (W2 D12 with its cotangents in the
            // workspace: 131 -> 98 KB, two teams of 256; W8 D4 FP64 forward:
            // 75 -> 42 KB, five teams of 128 instead of three)
            int m2 = mode | kTopGlobal;
            const size_t s2 = in.fp64 ? group_slice<double>(sg, t, m2, optin) : group_slice<float>(sg, t, m2, optin);
            const size_t fit = static_cast<size_t>(cta / t);
            if (s2 && std::min(fit, optin / s2) > std::min(fit, optin / slice)) {
                mode = m2;
                slice = s2;
            }
        }
        if (in.letters) {
            // forward-only, or forward + reverse (depth >= 3), in FP32 with
            // one warp per first letter
            const bool rev = job.mode & kBackward;
            if (in.fp64 || !(job.mode & kForward) || (!rev && !(job.mode & kTopLevel)) || t != 32 * in.g.width)
                return cudaErrorInvalidConfiguration;
            slice = rev ? letter_rev_slice_bytes(in.g.width, in.g.depth) : letter_slice_bytes(in.g.width, in.g.depth);
            if (slice == 0 || slice > optin) return cudaErrorInvalidConfiguration;
        }
        job.letters = in.letters ? 1 : 0;
        if (slice == 0) {
            *refusal = GroupRefusal::StateTooLarge;
            return cudaErrorNotSupported;
        }
        job.mode = mode;
        job.width = in.g.width;
        job.depth = in.g.depth;
        job.fp64 = in.fp64 ? 1 : 0;
        job.team_threads = static_cast<uint32_t>(t);
        job.slice = static_cast<uint32_t>(slice);
        job.teams = static_cast<uint32_t>(std::min<size_t>({static_cast<size_t>(cta / t), optin / slice,
                                                            static_cast<size_t>(kGroupMaxTeams)}));
        budget = std::max(budget, job.teams * slice);
        job.fd_m = in.g.divw.m;
        job.fd_l = in.g.divw.l;
        job.fault = in.g.fault;
        job.incr = in.incr;
        job.offsets = in.paths.offsets;
        job.length = in.paths.length;
        job.batch = in.paths.batch;
        job.sig = in.sig;
        job.sig_stride = in.sig_stride;
        job.seed = in.seed;
        job.seed_stride = in.seed_stride;
        job.grad = in.grad;
        // one increment's Chen-step FMAs, x4 with a reverse pass, x3 in FP64,
        // per thread of the team: the ordering key's weight
        int64_t f = 0;
        for (int i = 1; i <= in.g.depth; ++i) f += static_cast<int64_t>(in.g.depth - i + 1) * in.g.pw[i];
        job.weight = std::max<int64_t>(1, f * ((job.mode & kBackward) ? 4 : 1) * (in.fp64 ? 3 : 1) / t);
        if (in.paths.offsets && in.paths.batch > 0) ragged += in.paths.batch;
        if (in.paths.batch >= (int64_t{1} << 31)) {
            *refusal = GroupRefusal::TooManyPaths;
            return cudaErrorNotSupported;
        }
    }
    // with the launch's shared memory fixed, every job takes as many teams as fit
    for (int j = 0; j < njobs; ++j) {
        GroupJob& job = tab.job[j];
        job.teams = static_cast<uint32_t>(std::min<size_t>(
            {static_cast<size_t>(cta) / job.team_threads, budget / job.slice, static_cast<size_t>(kGroupMaxTeams)}));
        needed_ctas = std::max<int64_t>(needed_ctas, (job.batch + job.teams - 1) / job.teams);
    }
    if (needed_ctas == 0) return cudaSuccess;
    if ((err = allow_large_smem<kernel>(dev)) != cudaSuccess) return err;
    int per_sm = 0;
    if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, cta, budget)) != cudaSuccess)
        return err;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int64_t ctas = std::min<int64_t>(needed_ctas, static_cast<int64_t>(per_sm) * dev.sm_count);
    // scratch: the counters and the job sequence, the ragged orders, then the
    // cot jobs' workspaces (one slice per team of the launch; at W2 D12 FP64,
    // 98 KB a slice, 30 MB for two teams on each of 152 SMs: L2-resident)
    size_t ws_bytes = 0;
    const size_t orders_bytes = (static_cast<size_t>(ragged) * sizeof(int32_t) + 255) / 256 * 256;
    for (int j = 0; j < njobs; ++j) {
        GroupJob& job = tab.job[j];
        if (!job.cot) continue;
        const SigGeometry sg = make_sig_geometry(jobs[j].g);
        job.gws_stride = static_cast<int64_t>((sg.g.db[sg.g.depth] + sg.chain_total + 31) / 32 * 32);
        ws_bytes += static_cast<size_t>(ctas) * job.teams * job.gws_stride * sizeof(double);
    }
    void* scratch = nullptr;
    err = cudaMallocAsync(&scratch, 256 + orders_bytes + ws_bytes, s);
    if (err != cudaSuccess) return err;
    char* base = static_cast<char*>(scratch);
    tab.seq = reinterpret_cast<int32_t*>(base + 128);
    int32_t* order = reinterpret_cast<int32_t*>(base + 256);
    char* ws = base + 256 + orders_bytes;
    for (int j = 0; j < njobs; ++j) {
        GroupJob& job = tab.job[j];
        job.counter = reinterpret_cast<unsigned int*>(base) + j;
        if (job.offsets && job.batch > 0) {
            job.order = order;
            order += job.batch;
        }
        if (job.cot) {
            job.gws = ws;
            ws += static_cast<size_t>(ctas) * job.teams * job.gws_stride * sizeof(double);
        }
    }
    k_order_group<<<1, 1024, 0, s>>>(tab);
    err = cudaGetLastError();
    if (err == cudaSuccess) {
        kernel<<<dim3(static_cast<unsigned>(ctas)), cta, budget, s>>>(tab);
        err = cudaGetLastError();
    }
    cudaError_t ferr = cudaFreeAsync(scratch, s);
    return err != cudaSuccess ? err : ferr;
}

}  // namespace rpp_gb
