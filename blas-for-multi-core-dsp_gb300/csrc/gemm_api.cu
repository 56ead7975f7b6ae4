// gemm_api.cu -- gb_sgemm / gb_dgemm: argument checks, semantics and the
// per-shape choice of kernel.
//
// Covers the reference entry points sgemm_{NN,NT,TN,TT}_qxx
// (sgemm_release_V1.3.2/include/sgemm_kernel.h:11-22), dgemm_{NN,NT,TN,TT}
// (dgemm_release_V1.1/include/dgemm_kernel.h:39-60) and the irregular
// irr_{shortA,thinB}_{s,d}gemm_* (irr_*_kernel.h:11-22) behind one BLAS-style
// call; the transpose mode picks operand layouts, not separate drivers.
#include <string.h>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace gb {
namespace {

// C = beta*C (BLAS) / C = beta (scalar) / C = C + beta when K == 0.
template <typename T>
__global__ void k0_kernel(T *C, int64_t M, int64_t N, int64_t ldc, T beta, int semantics) {
    const int64_t total = M * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t m = e / N, n = e - m * N;
        T *cp = C + m * ldc + n;
        if (semantics == GB_SEM_BLAS)
            *cp = (beta == T(0)) ? T(0) : beta * *cp;
        else if (semantics == GB_SEM_SCALAR_BETA)
            *cp = T(0) + beta;
        else
            *cp = *cp + (T(0) + beta);
    }
}

template <typename T>
gb_status k0(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    int64_t total = g.M * g.N;
    int blocks = (int)(ceil_div(total, 256) < 8 * sm_count() ? ceil_div(total, 256) : 8 * sm_count());
    k0_kernel<T><<<blocks, 256, 0, g.stream>>>((T *)g.C, g.M, g.N, g.ldc, (T)g.beta, g.semantics);
    GB_LAUNCH_CHECK("k0_kernel");
    return ok();
}

// GB_ALGO_AUTO: skinny shapes stream through the skinny kernels; large FP32
// products go to 3xBF16 on tcgen05 once K is long enough for its
// representation error to sit inside 2*K*u32; large FP64 products go to the
// Ozaki slices (slice count chosen for FP64-level error), small ones stay on
// the bit-exact ordered DFMA kernel (GB300's FP64 pipe is ~1.2 TFLOP/s).
// (FP64 skinny products go to Ozaki too: native FP64 is ~1.2 TFLOP/s, and
// the slices of a very long K are processed in chunks of bounded workspace.)
int pick(int bits, bool ta, bool tb, int64_t M, int64_t N, int64_t K) {
    (void)ta; (void)tb;
    const int64_t small = M < N ? M : N;
    const int64_t large = M < N ? N : M;
    const double work = (double)M * (double)N * (double)K;
    if (bits == 64) {
        // FP64 skinny: the skinny path streams X once, cutting it into digits
        // for the tensor cores (the general Ozaki form would pad the small
        // side to 128 and re-read its slices for every slice pair)
        const bool skinny = small <= 64 && large >= 4 * small && large >= 1024;
        if (skinny) return GB_ALGO_SKINNY;
        if (work > 134217728.0) return GB_ALGO_OZAKI;   // 2^27 = 512^3
        return GB_ALGO_ORDERED;
    }
    // FP32 skinny: the skinny path streams X once (FFMA up to n = 8, 3xBF16
    // with X split in flight into tensor memory beyond)
    if (small <= 64 && large >= 4 * small && large >= 1024) return GB_ALGO_SKINNY;
    if (K >= 64 && work > 134217728.0) return GB_ALGO_BF16X3;
    return GB_ALGO_SIMT;
}

template <typename T>
gb_status run_algo(const GemmArgs &g, const gb_gemm_opts &o, const char *fn);

template <typename T>
gb_status gemm(char transA, char transB, int64_t M, int64_t N, int64_t K, T alpha, const T *A, int64_t lda,
               const T *B, int64_t ldb, T beta, T *C, int64_t ldc, const gb_gemm_opts *opts) {
    gb_gemm_opts o;
    if (opts) o = *opts; else gb_gemm_opts_init(&o);
    const char *fn = sizeof(T) == 8 ? "gb_dgemm" : "gb_sgemm";
    GB_CHECK_ARG(is_mode(transA) && is_mode(transB), "%s: transA/transB must be 'N' or 'T'", fn);
    GB_CHECK_ARG(M >= 0 && N >= 0 && K >= 0, "%s: negative dimension", fn);
    const bool ta = is_trans(transA), tb = is_trans(transB);
    const int64_t arows = ta ? K : M, acols = ta ? M : K;
    const int64_t brows = tb ? N : K, bcols = tb ? K : N;
    GB_CHECK_ARG(lda >= (acols > 1 ? acols : 1), "%s: lda (%lld) < %lld", fn, (long long)lda, (long long)acols);
    GB_CHECK_ARG(ldb >= (bcols > 1 ? bcols : 1), "%s: ldb (%lld) < %lld", fn, (long long)ldb, (long long)bcols);
    GB_CHECK_ARG(ldc >= (N > 1 ? N : 1), "%s: ldc (%lld) < N (%lld)", fn, (long long)ldc, (long long)N);
    GB_CHECK_ARG(o.semantics >= 0 && o.semantics <= 2, "%s: unknown semantics %d", fn, o.semantics);
    GB_CHECK_ARG(o.algo >= 0 && o.algo <= 8, "%s: unknown algo %d", fn, o.algo);
    GB_CHECK_ARG(o.k_block >= 0 && o.k_slab >= 0, "%s: negative k_block/k_slab", fn);
    GB_CHECK_ARG(o.split_k >= 0 && o.split_k <= 64, "%s: split_k %d not in 0..64", fn, o.split_k);
    if (M == 0 || N == 0) {
        if (!o.err_out) return ok();
        GemmArgs g0;
        g0.M = M; g0.N = N; g0.stream = as_stream(o.stream);
        return report_after(g0, sizeof(T) * 8, o.err_out);
    }
    GB_CHECK_ARG(C != nullptr, "%s: C is null", fn);
    if (K > 0) GB_CHECK_ARG(A != nullptr && B != nullptr, "%s: A or B is null", fn);
    (void)arows; (void)brows;

    GemmArgs g;
    g.ta = ta; g.tb = tb; g.M = M; g.N = N; g.K = K;
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = C; g.ldc = ldc;
    g.alpha = (double)alpha; g.beta = (double)beta;
    g.semantics = o.semantics;
    g.k_block = o.k_block; g.k_slab = o.k_slab; g.alpha_on_b = o.alpha_on_b;
    g.accum_k = o.accum_k; g.split_k = o.split_k;
    g.stream = as_stream(o.stream);
    if (!o.err_out) return run_algo<T>(g, o, fn);
    gb_status st = report_before(g, sizeof(T) * 8);
    if (st == GB_OK) st = run_algo<T>(g, o, fn);
    if (st == GB_OK) st = report_after(g, sizeof(T) * 8, o.err_out);
    return st;
}

// The product itself, with the algorithm the options ask for (AUTO picked by shape).
template <typename T>
gb_status run_algo(const GemmArgs &g, const gb_gemm_opts &o, const char *fn) {
    const bool ta = g.ta, tb = g.tb;
    const int64_t M = g.M, N = g.N, K = g.K;
    int algo = o.algo;
    if (algo == GB_ALGO_AUTO) algo = pick(sizeof(T) * 8, ta, tb, M, N, K);
    if (algo == GB_ALGO_ORDERED)
        return sizeof(T) == 8 ? launch_gemm_ordered_f64(g) : launch_gemm_ordered_f32(g);
    if (K == 0) return k0<T>(g);
    switch (algo) {
        case GB_ALGO_SIMT:
            return sizeof(T) == 8 ? launch_gemm_ordered_f64(g) : launch_sgemm_simt(g);
        case GB_ALGO_DMMA:
            if (sizeof(T) != 8) return set_status(GB_ERR_UNSUPPORTED, "gb_sgemm: DMMA is an FP64 algorithm");
            return launch_dgemm_dmma(g);
        case GB_ALGO_BF16X3:
            if (sizeof(T) != 4) return set_status(GB_ERR_UNSUPPORTED, "gb_dgemm: BF16X3 is an FP32 algorithm");
            return launch_sgemm_bf16x3(g);
        case GB_ALGO_BF16X6:
            if (sizeof(T) != 4) return set_status(GB_ERR_UNSUPPORTED, "gb_dgemm: BF16X6 is an FP32 algorithm");
            return launch_sgemm_bf16x6(g);
        case GB_ALGO_FP16X3:
            if (sizeof(T) != 4) return set_status(GB_ERR_UNSUPPORTED, "gb_dgemm: FP16X3 is an FP32 algorithm");
            return launch_sgemm_fp16x3(g);
        case GB_ALGO_OZAKI: {
            if (sizeof(T) != 8) return set_status(GB_ERR_UNSUPPORTED, "gb_sgemm: OZAKI is an FP64 algorithm");
            int s = o.ozaki_slices;
            GB_CHECK_ARG(s == 0 || (s >= 2 && s <= 9), "gb_dgemm: ozaki_slices %d not in 2..9", s);
            GB_CHECK_ARG(o.target_err >= 0.0, "gb_dgemm: negative target_err");
            if (s == 0) s = ozaki_pick_slices(o.target_err, K);
            return launch_dgemm_ozaki(g, s);
        }
        case GB_ALGO_SKINNY:
            return sizeof(T) == 8 ? launch_skinny_f64(g) : launch_skinny_f32(g);
        default:
            return set_status(GB_ERR_UNSUPPORTED, "%s: algo %d", fn, algo);
    }
}

}  // namespace

int resolve_algo(int bits, int algo, bool ta, bool tb, int64_t M, int64_t N, int64_t K) {
    return algo == GB_ALGO_AUTO ? pick(bits, ta, tb, M, N, K) : algo;
}

size_t gemm_workspace_bound(int bits, int algo, bool ta, bool tb, int64_t M, int64_t N, int64_t K, const void *A,
                            int64_t lda, const void *B, int64_t ldb, int slices, int split_k) {
    algo = resolve_algo(bits, algo, ta, tb, M, N, K);
    if (M <= 0 || N <= 0 || K <= 0) return 0;
    switch (algo) {
        case GB_ALGO_BF16X3:
        case GB_ALGO_BF16X6:
        case GB_ALGO_FP16X3: {   // two halves of pieces (up to three 16-bit pieces per operand) + line maxima
            const int64_t kp = ceil_div(K, 64) * 64;
            return 2 * ((size_t)3 * (M + N) * kp * 2 + (size_t)(M + N) * 4 + 1024) + 4096;
        }
        case GB_ALGO_SKINNY: {   // the skinny plan's own figure
            GemmArgs g;
            g.ta = ta; g.tb = tb; g.M = M; g.N = N; g.K = K;
            g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = nullptr; g.ldc = N;
            g.split_k = split_k;
            return skinny_workspace_bytes(g, bits);
        }
        case GB_ALGO_OZAKI: {   // slices of both operands (K cut into chunks past 4 GiB) + exponents
            const int s = slices > 0 ? slices : ozaki_pick_slices(0.0, K);
            const int64_t kp = ceil_div(K, 64) * 64, mp = ceil_div(M, 128) * 128, np = ceil_div(N, 256) * 256;
            double v = (double)s * (double)(mp + np) * (double)kp * 2.0;
            const double cap = 4.0 * (1ull << 30) + (double)s * (mp + np) * 1024 * 2.0;
            if (v > cap) v = cap;
            // + the wide form's FP64 scratch: 256 KB per CTA
            return (size_t)v + (size_t)(mp + np) * 4 + (size_t)sm_count() * (256 << 10) + 8192;
        }
        default:
            return 0;
    }
}

}  // namespace gb

extern "C" {

void gb_gemm_opts_init(gb_gemm_opts *opts) {
    if (!opts) return;
    memset(opts, 0, sizeof(*opts));
    opts->algo = GB_ALGO_AUTO;
    opts->semantics = GB_SEM_BLAS;
}

int gb_gemm_pick_algo(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K) {
    return gb::pick(dtype_bits, gb::is_trans(transA), gb::is_trans(transB), M, N, K);
}

gb_status gb_workspace_query(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                             const void *A, int64_t lda, const void *B, int64_t ldb, const gb_gemm_opts *opts,
                             size_t *bytes) {
    GB_CHECK_ARG(bytes != nullptr, "gb_workspace_query: bytes is NULL");
    *bytes = 0;
    GB_CHECK_ARG(dtype_bits == 32 || dtype_bits == 64, "gb_workspace_query: dtype_bits %d", dtype_bits);
    GB_CHECK_ARG(gb::is_mode(transA) && gb::is_mode(transB), "gb_workspace_query: transA/transB must be 'N' or 'T'");
    GB_CHECK_ARG(M >= 0 && N >= 0 && K >= 0, "gb_workspace_query: negative dimension");
    gb_gemm_opts o;
    if (opts) o = *opts;
    else gb_gemm_opts_init(&o);
    GB_CHECK_ARG(o.ozaki_slices == 0 || (o.ozaki_slices >= 2 && o.ozaki_slices <= 9),
                 "gb_workspace_query: ozaki_slices %d not in 2..9", o.ozaki_slices);
    GB_CHECK_ARG(o.target_err >= 0.0, "gb_workspace_query: negative target_err");
    const bool ta = gb::is_trans(transA), tb = gb::is_trans(transB);
    const int slices = o.ozaki_slices > 0 ? o.ozaki_slices : gb::ozaki_pick_slices(o.target_err, K);
    *bytes = gb::gemm_workspace_bound(dtype_bits, o.algo, ta, tb, M, N, K, A, lda, B, ldb, slices, o.split_k);
    return gb::ok();
}

gb_status gb_sgemm(char transA, char transB, int64_t M, int64_t N, int64_t K, float alpha, const float *A,
                   int64_t lda, const float *B, int64_t ldb, float beta, float *C, int64_t ldc,
                   const gb_gemm_opts *opts) {
    return gb::gemm<float>(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, opts);
}

gb_status gb_dgemm(char transA, char transB, int64_t M, int64_t N, int64_t K, double alpha, const double *A,
                   int64_t lda, const double *B, int64_t ldb, double beta, double *C, int64_t ldc,
                   const gb_gemm_opts *opts) {
    return gb::gemm<double>(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, opts);
}

}  // extern "C"
