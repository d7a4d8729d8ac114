/*
 * rpp_gb300.h -- C ABI of the GB300-native (sm_103a) batched free-tensor
 * library.  Plain pointers and sizes only: no CUDA, C++ or torch types cross
 * this boundary, so a ctypes / cgo / JNI caller binds it directly.
 *
 * The entry points are what RoughPathPrimitives' operation API calls through a
 * new `gpu` strategy (rpp::gpu::strategies::GB300Strategy, in the package's
 * include/rpp/gpu/gb300/strategy.hpp).  Each declaration names the reference
 * operation it replaces (paths relative to the reference project's root).
 *
 * Conventions (shared by every entry point):
 *  - Status codes are the reference's rpp::ErrorCode values
 *    (include/rpp/support/error.hpp:28-39); 0 is success.  The message of the
 *    last failure on the calling host thread is rpp_gb_last_error_string().
 *  - All tensor data pointers are DEVICE pointers.  A batch operand is
 *    {data, stride, min_degree, max_degree}: batch element b is the dense
 *    tensor at data + b*stride (elements, not bytes), coefficients in the
 *    graded lexicographic order of include/rpp/basis/tensor_basis.hpp; the
 *    degree range is the view's (include/rpp/views/dense_graded_vector_view.hpp):
 *    coefficients outside it read as zero and are never written.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    asynchronous and stream-ordered and none synchronises the device.  The
 *    per-operation entry points allocate nothing after their plan / matrix
 *    handle is created; rpp_gb_signature allocates stream-ordered scratch
 *    (cudaMallocAsync / cudaFreeAsync on `stream`) for ragged batches and for
 *    states larger than shared memory, and the fused Lie <-> tensor steps
 *    (rpp_gb_log_to_lie, rpp_gb_lie_to_tensor_exp) do the same for states
 *    larger than shared memory.
 *  - dtype selects the scalar and accumulation type: RPP_GB_F32 (float data,
 *    float accumulation) or RPP_GB_F64 (double, double).
 */
#ifndef RPP_GB300_H
#define RPP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* rpp::ErrorCode (include/rpp/support/error.hpp:28-39) */
enum rpp_gb_status {
    RPP_GB_SUCCESS = 0,
    RPP_GB_CANCELLED = 1,
    RPP_GB_UNKNOWN = 2,
    RPP_GB_INVALID_ARGUMENT = 3,
    RPP_GB_TIMEOUT = 4,
    RPP_GB_OUT_OF_RESOURCES = 5,
    RPP_GB_CONTRACT_VIOLATION = 6,
    RPP_GB_OUT_OF_BOUNDS = 7,
    RPP_GB_NOT_IMPLEMENTED = 8,
    RPP_GB_INTERNAL = 9
};

enum rpp_gb_dtype { RPP_GB_F32 = 0, RPP_GB_F64 = 1 };

/* rpp::ops::FTInplaceFMAType (include/rpp/operations/basic/ft_inplace_fma.hpp:17-21) */
enum rpp_gb_inplace_fma_kind {
    RPP_GB_A_EQUALS_BC_PLUS_A = 0, /* a <- alpha*a + beta*b(x)c */
    RPP_GB_A_EQUALS_AB_PLUS_C = 1, /* a <- alpha*c + beta*a(x)b */
    RPP_GB_A_EQUALS_BA_PLUS_C = 2  /* a <- alpha*c + beta*b(x)a */
};

/* rpp::ops::TensorAntipodeSigningPolicy (include/rpp/operations/basic/
 * tensor_generalised_antipode.hpp:14) */
enum rpp_gb_antipode_policy { RPP_GB_NO_SIGNING = 0, RPP_GB_SIGN_BY_DEGREE = 1 };

/* rpp::sparse::MatrixFormat (include/rpp/sparse/matrix.hpp:10-13) */
enum rpp_gb_matrix_format { RPP_GB_CSR = 0, RPP_GB_CSC = 1 };

typedef void* rpp_gb_stream;

typedef struct rpp_gb_plan rpp_gb_plan;
typedef struct rpp_gb_matrix rpp_gb_matrix;

typedef struct rpp_gb_tensor_arg {
    void* data;
    int64_t stride;
    int32_t min_degree;
    int32_t max_degree;
} rpp_gb_tensor_arg;

/* A graded vector operand of the sparse products, in begin-relative form:
 * element b's view starts at data + b*stride + begin and holds `size`
 * coefficients.  For a view over degrees [lo, hi] of a basis with table
 * degree_begin, begin = degree_begin[lo] and size = degree_begin[hi+1] - begin
 * (include/rpp/views/dense_graded_vector_view.hpp: begin()/size()). */
typedef struct rpp_gb_vector_arg {
    void* data;
    int64_t stride;
    int64_t begin;
    int64_t size;
} rpp_gb_vector_arg;

/* ------------------------------------------------------------------------
 * Plans.  A plan fixes (width, depth) and caches the device-side basis
 * tables the reference re-uploads on every launch (include/rpp/gpu/device.hpp:
 * 176-209 via include/rpp/basis/tensor_basis.hpp:104-117).  It is immutable
 * after creation and may be shared by concurrent calls on any streams.
 * width in [1, 255] (include/rpp/architecture.hpp:36-39), depth in [0, 30].
 * ---------------------------------------------------------------------- */
int rpp_gb_plan_create(rpp_gb_plan** plan, int32_t width, int32_t depth, int32_t device);
int rpp_gb_plan_destroy(rpp_gb_plan* plan);

/* Kernels stage operands with bulk copies completing on mbarriers and never
 * wait on them without a limit: a wait that runs out sets a bit in the plan's
 * fault word (1 = a bulk-copy wait expired; that launch's results are
 * invalid) and the kernel returns.  rpp_gb_plan_fault synchronises the plan's
 * device, returns the word and clears it (no reference counterpart).
 * rpp_gb_selftest_bounded_wait launches a one-CTA kernel whose wait is made to
 * expire (a transaction nothing completes, a short limit): afterwards
 * rpp_gb_plan_fault reports 1. */
int rpp_gb_plan_fault(const rpp_gb_plan* plan, uint32_t* fault);
int rpp_gb_selftest_bounded_wait(const rpp_gb_plan* plan, rpp_gb_stream stream);
const char* rpp_gb_last_error_string(void);
/* Library version, e.g. "rpp_gb300 1.0.0 sm_103a". */
const char* rpp_gb_version(void);

/* ------------------------------------------------------------------------
 * Free-tensor products.
 * ---------------------------------------------------------------------- */

/* rpp::ops::ft_mul (include/rpp/operations/basic/ft_mul.hpp:48-79):
 * out = beta * lhs (x) rhs on out's degree range. */
int rpp_gb_ft_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                  const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* lhs,
                  const rpp_gb_tensor_arg* rhs, int64_t batch, double beta);

/* rpp::ops::ft_fma (include/rpp/operations/basic/ft_fma.hpp:48-83):
 * out = alpha*a + beta * b (x) c. */
int rpp_gb_ft_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                  const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* a,
                  const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t batch,
                  double alpha, double beta);

/* rpp::ops::ft_inplace_fma<kind> (include/rpp/operations/basic/
 * ft_inplace_fma.hpp:64-96); `a` is read and written in place. */
int rpp_gb_ft_inplace_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          int32_t kind, const rpp_gb_tensor_arg* a, const rpp_gb_tensor_arg* b,
                          const rpp_gb_tensor_arg* c, int64_t batch, double alpha, double beta);

/* rpp::ops::ft_inplace_mul (include/rpp/operations/basic/ft_inplace_mul.hpp:
 * 40-69): lhs <- beta * lhs (x) rhs. */
int rpp_gb_ft_inplace_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          const rpp_gb_tensor_arg* lhs, const rpp_gb_tensor_arg* rhs,
                          int64_t batch, double beta);

/* rpp::ops::ft_exp (include/rpp/operations/intermediate/ft_exp.hpp:84-112). */
int rpp_gb_ft_exp(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                  const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* arg, int64_t batch);

/* rpp::ops::ft_fmexp (include/rpp/operations/intermediate/ft_fmexp.hpp:
 * 91-121): out = multiplier (x) exp(exponent); out must not alias multiplier. */
int rpp_gb_ft_fmexp(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                    const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* multiplier,
                    const rpp_gb_tensor_arg* exponent, int64_t batch);

/* rpp::ops::ft_log (include/rpp/operations/intermediate/ft_log.hpp:87-114). */
int rpp_gb_ft_log(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                  const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* arg, int64_t batch);

/* rpp::ops::ft_adj_lmul (include/rpp/operations/basic/ft_adj_lmul.hpp:44-73):
 * out[v] = sum_u op[u] arg[uv]. */
int rpp_gb_ft_adj_lmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                       const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op,
                       const rpp_gb_tensor_arg* arg, int64_t batch);

/* rpp::ops::ft_adj_rmul (include/rpp/operations/basic/ft_adj_rmul.hpp:42-71):
 * out[u] = sum_v op[v] arg[uv]. */
int rpp_gb_ft_adj_rmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                       const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op,
                       const rpp_gb_tensor_arg* arg, int64_t batch);

/* rpp::ops::tensor_generalised_antipode<policy> (include/rpp/operations/
 * basic/tensor_generalised_antipode.hpp:42-69); tensor_antipode and
 * tensor_reflect are the two policies. */
int rpp_gb_tensor_antipode(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                           int32_t policy, const rpp_gb_tensor_arg* out,
                           const rpp_gb_tensor_arg* arg, int64_t batch);

/* Helper ops composed inside the intermediate operations:
 * rpp::ops::vector_assign (include/rpp/operations/linalg/vector_assign.hpp),
 * vector_set_constant (vector_set_constant.hpp), tensor_set_identity and
 * tensor_add_identity (include/rpp/operations/basic/tensor_*_identity.hpp). */
int rpp_gb_vector_assign(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                         const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* arg,
                         int64_t batch);
int rpp_gb_vector_set_constant(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                               const rpp_gb_tensor_arg* out, int64_t batch, double value);
int rpp_gb_tensor_set_identity(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                               const rpp_gb_tensor_arg* out, int64_t batch, double scalar);
int rpp_gb_tensor_add_identity(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                               const rpp_gb_tensor_arg* out, int64_t batch, double scalar);

/* ------------------------------------------------------------------------
 * Shuffle algebra and the tensor pairing.  A coefficient of degree n of a
 * shuffle product sums 2^n terms (word_shuffle_product.hpp:43-97); terms whose
 * factors lie outside an operand's degree range are omitted, never read.
 * ---------------------------------------------------------------------- */

/* rpp::ops::st_mul (include/rpp/operations/basic/st_mul.hpp:53-79):
 * out = beta * lhs sh rhs on out's degree range. */
int rpp_gb_st_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                  const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* lhs,
                  const rpp_gb_tensor_arg* rhs, int64_t batch, double beta);

/* rpp::ops::st_fma (include/rpp/operations/basic/st_fma.hpp:56-85):
 * out = alpha*a + beta * b sh c. */
int rpp_gb_st_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                  const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* a,
                  const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t batch,
                  double alpha, double beta);

/* rpp::ops::st_inplace_fma (include/rpp/operations/basic/st_inplace_fma.hpp:
 * 50-80): a <- alpha*a + beta * b sh c.  a must not overlap b or c. */
int rpp_gb_st_inplace_fma(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          const rpp_gb_tensor_arg* a, const rpp_gb_tensor_arg* b,
                          const rpp_gb_tensor_arg* c, int64_t batch, double alpha, double beta);

/* rpp::ops::st_adj_mul (include/rpp/operations/basic/st_adj_mul.hpp:46-69):
 * the adjoint of x -> op sh x, out[w] = sum_u op[u] sum_{s in w sh u} arg[s].
 * Every coefficient of out's range is written (zero when no term exists). */
int rpp_gb_st_adj_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                      const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op,
                      const rpp_gb_tensor_arg* arg, int64_t batch);

/* rpp::ops::left_hs_mul (include/rpp/operations/basic/left_hs_mul.hpp:59-87):
 * out = beta * integrator < integrand (left half-shuffle; the first letter
 * of every word comes from the integrator), out[0] = 0. */
int rpp_gb_left_hs_mul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                       const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* integrator,
                       const rpp_gb_tensor_arg* integrand, int64_t batch, double beta);

/* rpp::ops::left_hs_adj_lmul (include/rpp/operations/basic/
 * left_hs_adj_lmul.hpp:39-57): the adjoint of y -> x < y with x = op (the
 * integrator) fixed and arg the cotangent:
 * out[w] = beta * sum_a sum_u op[a u] sum_{s in w sh u} arg[a s].
 * beta scales the result as in the reference's block strategy (its CPU
 * strategy takes no scale: beta = 1). */
int rpp_gb_left_hs_adj_lmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                            const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op,
                            const rpp_gb_tensor_arg* arg, int64_t batch, double beta);

/* rpp::ops::left_hs_adj_rmul (include/rpp/operations/basic/
 * left_hs_adj_rmul.hpp:39-57): the adjoint of x -> x < y with op the
 * cotangent (integrator slot) and arg = y (the integrand) fixed:
 * out[a v] = beta * sum_u arg[u] sum_{s in v sh u} op[a s], out[0] = 0. */
int rpp_gb_left_hs_adj_rmul(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                            const rpp_gb_tensor_arg* out, const rpp_gb_tensor_arg* op,
                            const rpp_gb_tensor_arg* arg, int64_t batch, double beta);

/* rpp::ops::tensor_pairing (include/rpp/operations/basic/tensor_pairing.hpp:
 * 47-73): result[b] = sum of functional[i] arg[i] over the degrees both views
 * hold (0 when they share none).  `result` is a device array of `batch`
 * contiguous scalars of dtype (rpp::make_scalar_batch,
 * include/rpp/views/scalar_view.hpp:53-60). */
int rpp_gb_tensor_pairing(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          void* result, const rpp_gb_tensor_arg* functional,
                          const rpp_gb_tensor_arg* arg, int64_t batch);

/* ------------------------------------------------------------------------
 * Sparse matrices and the Lie <-> tensor conversions.
 * ---------------------------------------------------------------------- */

/* Upload a host compressed matrix once (the reference maps it to the device on
 * every launch: include/rpp/sparse/detail/compressed_matrix.hpp:157-203).
 * outer_dim/inner_dim/offsets/indices follow rpp::sparse::CompressedMatrix
 * (compressed_matrix.hpp:38-125): CSR outer = rows, CSC outer = columns.  A
 * CSC matrix is transposed to CSR here (the reference's swap_format,
 * compressed_matrix.hpp:675-744), so products are atomic-free and
 * deterministic.  Values are stored in both precisions. */
int rpp_gb_matrix_create(rpp_gb_matrix** matrix, int32_t format, int64_t outer_dim,
                         int64_t inner_dim, int64_t nnz, const int64_t* offsets,
                         const int64_t* indices, const double* values, int32_t device);
int rpp_gb_matrix_destroy(rpp_gb_matrix* matrix);
/* The fault word of the sparse products run with this matrix (the same bits
 * as rpp_gb_plan_fault): synchronises the device, returns and clears it. */
int rpp_gb_matrix_fault(const rpp_gb_matrix* matrix, uint32_t* fault);

/* rpp::ops::sparse_matrix_vector_product (include/rpp/operations/linalg/
 * sparse_matrix_vector.hpp:57-96) with the CPU strategy's begin-relative
 * indexing (include/rpp/cpu/single_thread/operations/linalg/
 * sparse_matrix_vector.hpp:57-86, :138-163), batched as one SpMM:
 * out.begin()[r] = alpha * sum_c M[r][c] arg.begin()[c].  When the matrix was
 * created from CSC, the whole out view is zeroed first as the CSC product
 * does; a CSR product writes rows [0, rows) only.  This is also
 * rpp::ops::tensor_to_lie / lie_to_tensor (include/rpp/operations/basic/
 * tensor_to_lie.hpp:65-103, lie_to_tensor.hpp:70-108). */
int rpp_gb_sparse_matrix_vector(const rpp_gb_matrix* matrix, rpp_gb_stream stream,
                                int32_t dtype, const rpp_gb_vector_arg* out,
                                const rpp_gb_vector_arg* arg, int64_t batch, double alpha);

/* Fused steps either side of the signature.  Neither has a reference
 * counterpart as one call: each computes the composition named below without
 * writing the intermediate tensor to global memory.  The matrix handle must
 * live on the plan's device; the tensor view [min_degree, max_degree] is
 * clipped to the plan's depth. */

/* rpp::ops::ft_log (include/rpp/operations/intermediate/ft_log.hpp:87-114)
 * of `arg` into a tensor view over degrees [min_degree, max_degree], then
 * rpp::ops::tensor_to_lie (include/rpp/operations/basic/tensor_to_lie.hpp:
 * 65-103) with that view as the argument, i.e. rpp_gb_sparse_matrix_vector
 * with arg = {log, begin = degree_begin[min_degree], size = degree_begin[
 * max_degree+1] - begin}: out.begin()[r] = alpha * sum_c M[r][c] log[begin+c].
 * With the tensor_to_lie matrix and a full view this is the log-signature. */
int rpp_gb_log_to_lie(const rpp_gb_plan* plan, const rpp_gb_matrix* matrix, rpp_gb_stream stream,
                      int32_t dtype, const rpp_gb_vector_arg* out, const rpp_gb_tensor_arg* arg,
                      int32_t min_degree, int32_t max_degree, int64_t batch, double alpha);

/* rpp::ops::lie_to_tensor (include/rpp/operations/basic/lie_to_tensor.hpp:
 * 70-108) of `arg` into degrees [min_degree, max_degree] of a zero tensor X
 * (X.begin()[r] = alpha * sum_c M[r][c] arg.begin()[c]), then
 * rpp::ops::ft_exp (include/rpp/operations/intermediate/ft_exp.hpp) of X into
 * `out` when `multiplier` is NULL, else rpp::ops::ft_fmexp (ft_fmexp.hpp:
 * 91-121): out = multiplier (x) exp(X); out must not alias multiplier.  With
 * the lie_to_tensor matrix this is one step of a path given by Lie
 * increments. */
int rpp_gb_lie_to_tensor_exp(const rpp_gb_plan* plan, const rpp_gb_matrix* matrix, rpp_gb_stream stream,
                             int32_t dtype, const rpp_gb_tensor_arg* out,
                             const rpp_gb_tensor_arg* multiplier, const rpp_gb_vector_arg* arg,
                             int32_t min_degree, int32_t max_degree, int64_t batch, double alpha);

/* Hall basis and conversion matrices built natively (restating
 * include/rpp/basis/hall_basis.hpp:35-88, include/rpp/basis/
 * lie_multiplication.hpp:163-251, include/rpp/sparse/t2l_matrix.hpp:57-142 and
 * include/rpp/sparse/l2t_matrix.hpp:58-114, bit-exact).  Query sizes with NULL
 * outputs first: rpp_gb_lie_basis returns true_size in *true_size and fills
 * degree_begin (depth+2) and pairs (2*true_size) when non-NULL;
 * rpp_gb_conversion_matrix fills a CSC matrix (which = 0: tensor_to_lie,
 * which = 1: lie_to_tensor) when the arrays are non-NULL. */
int rpp_gb_lie_basis(int32_t width, int32_t depth, int64_t* true_size, int64_t* degree_begin,
                     int64_t* pairs);
int rpp_gb_conversion_matrix(int32_t width, int32_t depth, int32_t which, int64_t* outer_dim,
                             int64_t* inner_dim, int64_t* nnz, int64_t* offsets,
                             int64_t* indices, double* values);

/* ------------------------------------------------------------------------
 * Signatures of piecewise-linear paths (no reference counterpart as one
 * call: the reference caller loops ft_fmexp once per increment,
 * tests/rpp/gpu/block/ops/ft_fmexp_tests.cu:126-147).
 *
 * Increments are a packed ragged array: path b owns increments
 * [offsets[b], offsets[b+1]) of `incr` (each `width` scalars, row-major).
 * `offsets` is a DEVICE array of batch+1 int64; pass NULL with `length` > 0
 * for equal-length paths (offsets[b] = b*length).
 *
 * rpp_gb_signature: sig[b] (stride sig_stride) = S(x_b) =
 *   exp(dx_1) (x) ... (x) exp(dx_L), from the unit tensor.  When seed and
 * grad are non-NULL the same launch also runs the reverse pass and writes
 *   grad[k] = d/d(dx_k) sum_b <seed_b, S(x_b)>
 * (seed b at seed + b*seed_stride), recomputing prefixes backwards by
 * S_{k-1} = S_k (x) exp(-dx_k) instead of storing them.  sig may be NULL
 * when only the gradient is wanted.
 *
 * rpp_gb_signature_backward: the reverse pass alone, from final signatures
 * `sig` (as produced by rpp_gb_signature) and cotangents `seed`.
 * ---------------------------------------------------------------------- */
int rpp_gb_signature(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                     const void* incr, const int64_t* offsets, int64_t length, int64_t batch,
                     void* sig, int64_t sig_stride, const void* seed, int64_t seed_stride,
                     void* grad);
int rpp_gb_signature_backward(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                              const void* incr, const int64_t* offsets, int64_t length,
                              int64_t batch, const void* sig, int64_t sig_stride,
                              const void* seed, int64_t seed_stride, void* grad);

/* rpp_gb_signature over HOST buffers (no counterpart in the reference), for
 * callers whose paths live in host memory: incr, sig, seed and grad are host
 * pointers (same layouts and strides as rpp_gb_signature; equal-length paths
 * only, length > 0).  The batch is processed in chunks of `chunk` paths (0:
 * two chunks) that alternate between two internal streams; on each, a chunk
 * is copied in, computed with the schedule recorded for this shape and copied
 * out, so one chunk's copies overlap another chunk's kernels.  Pinned host
 * memory lets the copies run asynchronously (pageable memory works but
 * serialises them).  Stream-ordered: the internal streams start after the work
 * already on `stream`, and `stream` waits for them, so the host outputs are
 * complete once `stream` has passed the call (e.g. after
 * cudaStreamSynchronize).  Device buffers for two chunks are allocated
 * stream-ordered and released at the end.  The results equal
 * rpp_gb_signature's on device copies of the same arrays. */
int rpp_gb_signature_host(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          const void* incr, int64_t length, int64_t batch, void* sig,
                          int64_t sig_stride, const void* seed, int64_t seed_stride,
                          void* grad, int64_t chunk);

/* rpp_gb_signature without any device allocation (no counterpart in the
 * reference).  For callers that cannot allocate device memory at call time:
 * runtimes that own all device memory through their own allocator and forbid
 * cudaMalloc / cudaMallocAsync from plugins, real-time loops that must not wait
 * on or grow a memory pool, and hosts that budget device memory up front.
 * Same arguments, results and numerics as rpp_gb_signature; the only scratch
 * it needs (the work counter and longest-first order of a ragged batch) lives
 * in a fixed 8 MiB device array of the library, held by every GPU that loads
 * the library until the process exits.  Limits: a ragged batch of at most
 * 2,097,088 paths (RPP_GB_OUT_OF_BOUNDS beyond), and only shapes whose state
 * fits one CTA's shared memory (RPP_GB_NOT_IMPLEMENTED otherwise, e.g. width 6
 * depth 6 in FP64).  All calls share the array and it keeps the previous
 * call's contents (each call re-initialises what it reads), so calls whose
 * launches may overlap on the GPU race and must be serialised by the caller.
 * A schedule recorded by rpp_gb_signature_tune for the same shape is used,
 * except that a launch it gives a cotangent workspace (bit 26, an
 * allocation) keeps its cotangent arrays in shared memory instead; a schedule
 * whose launch would need a workspace is refused before anything is launched.
 * The first call on each device looks up the array's device address (with
 * that device current) and keeps it for the life of the process, which
 * assumes the device's context is not destroyed while the library is in use;
 * make that first call before any stream capture. */
int rpp_gb_signature_static_scratch(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                                    const void* incr, const int64_t* offsets, int64_t length,
                                    int64_t batch, void* sig, int64_t sig_stride, const void* seed,
                                    int64_t seed_stride, void* grad);

/* Autotuner for rpp_gb_signature (no reference counterpart): runs the same
 * call once per candidate schedule (threads per CTA of the shared-memory
 * kernel; optionally fewer CTAs per SM than fit, which trades occupancy for a
 * fuller last wave; for forward+reverse calls with signature output, also
 * the same work as a forward launch followed by a reverse launch from the
 * final signatures, each holding less shared memory per CTA) on the caller's
 * own inputs, times each with CUDA events on `stream`, and records the
 * fastest for this (device, width, depth, dtype, outputs requested, ragged or
 * not); later rpp_gb_signature calls with that key use it.  Synchronises the
 * stream (not capturable); leaves the chosen schedule's outputs in sig/grad.
 * *threads and *ms (may be NULL) receive the choice and its time per call:
 * threads per CTA in bits 0-9 of *threads, the cap on CTAs per SM (0 = none)
 * in bits 10-13, bit 14 set for the two-launch form, bit 15 set when its
 * forward launch (or a forward-only call) keeps the top level in the output
 * row in global memory, and
 * for the two-launch form the reverse launch's own CTA size in bits 16-25
 * (0: the same as the forward launch's), and bit 26 set when the launch with
 * the reverse pass keeps the cotangent arrays in a global workspace (the
 * state and forward chains stay in shared memory; more CTAs per SM for deep
 * narrow shapes), bit 27 set for the reverse step with D barriers instead of
 * 2D-1, and P-1 in bits 28-30 when each path's state is split over a
 * thread-block cluster of P CTAs by first letter (P divides the width; one
 * fused launch; bit 15 then puts the top level in the signature and seed
 * rows) -- tried for states whose tensor exceeds 48 KB.  In FP32, bit 16
 * without bit 14 selects the kernels with one warp per first letter and
 * compile-time (width, depth) (forward-only, and forward + reverse for depth
 * >= 3), which FP32 calls of their shapes take when no schedule is recorded.
 * A two-launch winner
 * is refined by timing other reverse sizes, then other forward sizes, and the
 * three fastest schedules with a reverse pass are timed with bit 27 too. */
int rpp_gb_signature_tune(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          const void* incr, const int64_t* offsets, int64_t length, int64_t batch,
                          void* sig, int64_t sig_stride, const void* seed, int64_t seed_stride,
                          void* grad, int32_t* threads, float* ms);

/* rpp_gb_signature under an explicit schedule (encoded as *threads of
 * rpp_gb_signature_tune), once, without consulting or changing the recorded
 * choice: for pinning a schedule and for testing every schedule. */
int rpp_gb_signature_with_schedule(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                                   const void* incr, const int64_t* offsets, int64_t length,
                                   int64_t batch, void* sig, int64_t sig_stride, const void* seed,
                                   int64_t seed_stride, void* grad, int32_t schedule);

/* Several signature calls in ONE persistent launch (no reference
 * counterpart: the reference launches ft_fmexp once per increment and per
 * shape).  Each job carries the arguments of one rpp_gb_signature call -- its
 * plan (width, depth), dtype, equal-length or ragged increments, outputs --
 * so one launch covers batches of different (width, depth) and of FP64 and
 * FP32 together, e.g. inside one captured CUDA graph.  Each path of job j is
 * run by a team of `threads` threads (bits 0-9: a multiple of 32, at least
 * width*depth; 0: for FP32 jobs of the shapes of the warp-per-letter kernels
 * (rpp_gb_signature_tune's bit 16) a team of width warps running that code,
 * otherwise the CTA size of the schedule recorded for that shape by
 * rpp_gb_signature_tune, else a heuristic; bit 26, or a recorded one-launch
 * schedule with bit 26, on an FP64 forward + reverse job: its cotangent level
 * and chains in a stream-ordered global workspace, one slice per team, so
 * more teams of a deep state fit per SM); a CTA holds as many teams of the
 * job in progress as its threads and shared memory allow, so small states
 * keep many paths per SM beside large ones.  CTAs take the jobs in order of
 * their most expensive path and, inside a job, paths longest first from a
 * work counter.  Each job's outputs equal, bit for bit, those of a separate
 * rpp_gb_signature call with `threads` threads per CTA (and the same
 * reverse-step form and cotangent placement).  `schedule`: threads per CTA in bits 0-9 (at most 640;
 * 0: 640) and bit 27 for the D-barrier reverse step.  Limits: 1 to 8 jobs,
 * all plans on one device, each job's state in one team's shared memory
 * (RPP_GB_NOT_IMPLEMENTED otherwise, e.g. width 6 depth 6 in FP64: run it
 * with rpp_gb_signature), fewer than 2^31 paths per job.  Stream-ordered;
 * the job order, work counters and cotangent workspaces are allocated
 * stream-ordered and released after the launch. */
typedef struct rpp_gb_signature_job {
    const rpp_gb_plan* plan;
    int32_t dtype;
    int32_t threads;
    const void* incr;
    const int64_t* offsets;
    int64_t length;
    int64_t batch;
    void* sig;
    int64_t sig_stride;
    const void* seed;
    int64_t seed_stride;
    void* grad;
} rpp_gb_signature_job;
int rpp_gb_signature_group(rpp_gb_stream stream, const rpp_gb_signature_job* jobs, int32_t njobs,
                           int32_t schedule);

/* Vector-Jacobian product of exp for a degree-one argument (no reference
 * counterpart; it closes the stored-prefix reverse pass composed from
 * ft_fmexp, ft_exp, ft_adj_lmul and ft_adj_rmul): for batch element b with
 * letters x[b*x_stride .. +width) and cotangent H (tensor, stride
 * cotangent_stride) of E = exp(x), writes dx_a = sum_w H[w] dE[w]/dx_a to
 * dx[b*dx_stride + a]. */
int rpp_gb_exp_letter_vjp(const rpp_gb_plan* plan, rpp_gb_stream stream, int32_t dtype,
                          const void* cotangent, int64_t cotangent_stride, const void* x,
                          int64_t x_stride, void* dx, int64_t dx_stride, int64_t batch);

/* ------------------------------------------------------------------------
 * Diagnostics (no reference counterpart).
 * rpp_gb_fma_peak: measured FMA throughput of `device` in TFLOP/s (2 flops per
 * FMA) for dtype, from a short dependent-chain kernel; the benchmark uses it
 * as the roofline denominator of the FMA-bound kernels.  Allocates a small
 * scratch buffer and synchronises the device.
 * ---------------------------------------------------------------------- */
int rpp_gb_fma_peak(int32_t dtype, int32_t device, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* RPP_GB300_H */
