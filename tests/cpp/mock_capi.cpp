// Test double of the C ABI (include/rpp_gb300.h): records each call's
// arguments as one text line so the strategy test can check how the
// GB300Strategy specialisations translate reference batches.  No GPU needed.
#include <cstdio>
#include <string>

#include <rpp_gb300.h>

std::string g_calls;
static char g_buf[512];
static int g_plan_dummy, g_matrix_dummy;

static void rec(const char* name, const rpp_gb_tensor_arg* a) {
    std::snprintf(g_buf, sizeof g_buf, " %s{s=%lld,%d..%d}", name, (long long)a->stride, a->min_degree, a->max_degree);
    g_calls += g_buf;
}
static void head(const char* op, int32_t dtype, int64_t n) {
    std::snprintf(g_buf, sizeof g_buf, "%s dtype=%d n=%lld", op, dtype, (long long)n);
    g_calls += g_buf;
}
static void tail(double a, double b) {
    std::snprintf(g_buf, sizeof g_buf, " a=%g b=%g\n", a, b);
    g_calls += g_buf;
}

extern "C" {
int rpp_gb_plan_create(rpp_gb_plan** plan, int32_t w, int32_t d, int32_t dev) {
    std::snprintf(g_buf, sizeof g_buf, "plan_create W=%d D=%d dev=%d\n", w, d, dev);
    g_calls += g_buf;
    *plan = reinterpret_cast<rpp_gb_plan*>(&g_plan_dummy);
    return 0;
}
int rpp_gb_plan_destroy(rpp_gb_plan*) { return 0; }
const char* rpp_gb_last_error_string(void) { return "mock"; }
const char* rpp_gb_version(void) { return "mock"; }
int rpp_gb_ft_mul(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* o, const rpp_gb_tensor_arg* l,
                  const rpp_gb_tensor_arg* r, int64_t n, double beta) {
    head("ft_mul", t, n); rec("out", o); rec("lhs", l); rec("rhs", r); tail(0, beta); return 0;
}
int rpp_gb_ft_fma(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* o, const rpp_gb_tensor_arg* a,
                  const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t n, double al, double be) {
    head("ft_fma", t, n); rec("out", o); rec("a", a); rec("b", b); rec("c", c); tail(al, be); return 0;
}
int rpp_gb_ft_inplace_fma(const rpp_gb_plan*, rpp_gb_stream, int32_t t, int32_t kind, const rpp_gb_tensor_arg* a,
                          const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t n, double al, double be) {
    head("ft_inplace_fma", t, n);
    std::snprintf(g_buf, sizeof g_buf, " kind=%d", kind); g_calls += g_buf;
    rec("a", a); rec("b", b); rec("c", c); tail(al, be); return 0;
}
int rpp_gb_ft_inplace_mul(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* l,
                          const rpp_gb_tensor_arg* r, int64_t n, double be) {
    head("ft_inplace_mul", t, n); rec("lhs", l); rec("rhs", r); tail(0, be); return 0;
}
#define UNARY(NAME)                                                                                   \
    int rpp_gb_##NAME(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* o,     \
                      const rpp_gb_tensor_arg* a, int64_t n) {                                      \
        head(#NAME, t, n); rec("out", o); rec("arg", a); tail(0, 0); return 0;                        \
    }
UNARY(ft_exp)
UNARY(ft_log)
UNARY(vector_assign)
#define BINARY(NAME)                                                                                  \
    int rpp_gb_##NAME(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* o,     \
                      const rpp_gb_tensor_arg* x, const rpp_gb_tensor_arg* y, int64_t n) {          \
        head(#NAME, t, n); rec("out", o); rec("x", x); rec("y", y); tail(0, 0); return 0;             \
    }
BINARY(ft_fmexp)
BINARY(ft_adj_lmul)
BINARY(ft_adj_rmul)
BINARY(st_adj_mul)
#define SCALED(NAME)                                                                                  \
    int rpp_gb_##NAME(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* o,     \
                      const rpp_gb_tensor_arg* x, const rpp_gb_tensor_arg* y, int64_t n, double b) { \
        head(#NAME, t, n); rec("out", o); rec("x", x); rec("y", y); tail(0, b); return 0;             \
    }
SCALED(st_mul)
SCALED(left_hs_mul)
SCALED(left_hs_adj_lmul)
SCALED(left_hs_adj_rmul)
int rpp_gb_st_fma(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* o, const rpp_gb_tensor_arg* a,
                  const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t n, double al, double be) {
    head("st_fma", t, n); rec("out", o); rec("a", a); rec("b", b); rec("c", c); tail(al, be); return 0;
}
int rpp_gb_st_inplace_fma(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* a,
                          const rpp_gb_tensor_arg* b, const rpp_gb_tensor_arg* c, int64_t n, double al, double be) {
    head("st_inplace_fma", t, n); rec("a", a); rec("b", b); rec("c", c); tail(al, be); return 0;
}
int rpp_gb_log_to_lie(const rpp_gb_plan*, const rpp_gb_matrix*, rpp_gb_stream, int32_t t, const rpp_gb_vector_arg* o,
                      const rpp_gb_tensor_arg* a, int32_t lo, int32_t hi, int64_t n, double alpha) {
    head("log_to_lie", t, n);
    std::snprintf(g_buf, sizeof g_buf, " out{b=%lld,n=%lld} degrees=%d..%d", (long long)o->begin, (long long)o->size,
                  lo, hi);
    g_calls += g_buf;
    rec("arg", a); tail(alpha, 0); return 0;
}
int rpp_gb_lie_to_tensor_exp(const rpp_gb_plan*, const rpp_gb_matrix*, rpp_gb_stream, int32_t t,
                             const rpp_gb_tensor_arg* o, const rpp_gb_tensor_arg* mult, const rpp_gb_vector_arg* a,
                             int32_t lo, int32_t hi, int64_t n, double alpha) {
    head("lie_to_tensor_exp", t, n); rec("out", o);
    if (mult) rec("mult", mult);
    std::snprintf(g_buf, sizeof g_buf, " arg{b=%lld,n=%lld} degrees=%d..%d", (long long)a->begin, (long long)a->size,
                  lo, hi);
    g_calls += g_buf;
    tail(alpha, 0); return 0;
}
int rpp_gb_tensor_pairing(const rpp_gb_plan*, rpp_gb_stream, int32_t t, void* result, const rpp_gb_tensor_arg* f,
                          const rpp_gb_tensor_arg* a, int64_t n) {
    head("tensor_pairing", t, n);
    std::snprintf(g_buf, sizeof g_buf, " result=%s", result ? "set" : "null"); g_calls += g_buf;
    rec("f", f); rec("arg", a); tail(0, 0); return 0;
}
int rpp_gb_tensor_antipode(const rpp_gb_plan*, rpp_gb_stream, int32_t t, int32_t policy, const rpp_gb_tensor_arg* o,
                           const rpp_gb_tensor_arg* a, int64_t n) {
    head("tensor_antipode", t, n);
    std::snprintf(g_buf, sizeof g_buf, " policy=%d", policy); g_calls += g_buf;
    rec("out", o); rec("arg", a); tail(0, 0); return 0;
}
#define FILL(NAME)                                                                                    \
    int rpp_gb_##NAME(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const rpp_gb_tensor_arg* o,     \
                      int64_t n, double v) {                                                        \
        head(#NAME, t, n); rec("out", o); tail(v, 0); return 0;                                       \
    }
FILL(vector_set_constant)
FILL(tensor_set_identity)
FILL(tensor_add_identity)
int rpp_gb_matrix_create(rpp_gb_matrix** m, int32_t fmt, int64_t outer, int64_t inner, int64_t nnz, const int64_t*,
                         const int64_t*, const double*, int32_t dev) {
    std::snprintf(g_buf, sizeof g_buf, "matrix_create fmt=%d outer=%lld inner=%lld nnz=%lld dev=%d\n", fmt,
                  (long long)outer, (long long)inner, (long long)nnz, dev);
    g_calls += g_buf;
    *m = reinterpret_cast<rpp_gb_matrix*>(&g_matrix_dummy);
    return 0;
}
int rpp_gb_matrix_destroy(rpp_gb_matrix*) { return 0; }
int rpp_gb_sparse_matrix_vector(const rpp_gb_matrix*, rpp_gb_stream, int32_t t, const rpp_gb_vector_arg* o,
                                const rpp_gb_vector_arg* a, int64_t n, double alpha) {
    head("spmv", t, n);
    std::snprintf(g_buf, sizeof g_buf, " out{s=%lld,begin=%lld,size=%lld} arg{s=%lld,begin=%lld,size=%lld}",
                  (long long)o->stride, (long long)o->begin, (long long)o->size, (long long)a->stride,
                  (long long)a->begin, (long long)a->size);
    g_calls += g_buf;
    tail(alpha, 0);
    return 0;
}
int rpp_gb_lie_basis(int32_t, int32_t, int64_t*, int64_t*, int64_t*) { return 0; }
int rpp_gb_conversion_matrix(int32_t, int32_t, int32_t, int64_t*, int64_t*, int64_t*, int64_t*, int64_t*, double*) {
    return 0;
}
int rpp_gb_signature(const rpp_gb_plan*, rpp_gb_stream, int32_t t, const void*, const int64_t* offsets, int64_t len,
                     int64_t n, void*, int64_t ss, const void* seed, int64_t, void* grad) {
    head("signature", t, n);
    std::snprintf(g_buf, sizeof g_buf, " len=%lld offsets=%d sig_stride=%lld seed=%d grad=%d\n", (long long)len,
                  offsets != nullptr, (long long)ss, seed != nullptr, grad != nullptr);
    g_calls += g_buf;
    return 0;
}
int rpp_gb_signature_backward(const rpp_gb_plan*, rpp_gb_stream, int32_t, const void*, const int64_t*, int64_t,
                              int64_t, const void*, int64_t, const void*, int64_t, void*) {
    return 0;
}
int rpp_gb_fma_peak(int32_t, int32_t, double*) { return 0; }
int rpp_gb_signature_static_scratch(const rpp_gb_plan*, rpp_gb_stream, int32_t, const void*, const int64_t*, int64_t,
                                    int64_t, void*, int64_t, const void*, int64_t, void*) {
    return 0;
}
int rpp_gb_signature_tune(const rpp_gb_plan*, rpp_gb_stream, int32_t, const void*, const int64_t*, int64_t, int64_t,
                          void*, int64_t, const void*, int64_t, void*, int32_t*, float*) {
    return 0;
}
int rpp_gb_exp_letter_vjp(const rpp_gb_plan*, rpp_gb_stream, int32_t, const void*, int64_t, const void*, int64_t,
                          void*, int64_t, int64_t) {
    return 0;
}
}
