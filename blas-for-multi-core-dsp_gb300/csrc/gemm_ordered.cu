// gemm_ordered.cu -- GEMM in the reference's summation order, bit-exact.
//
// Every C element is computed exactly as the reference's host check loop
// computes it, so results are bit-identical to those loops:
//   two-level sum (dgemm_release_V1.1/host_code/dgemm_demo.c:233-252,
//   sgemm_release_V1.3.2/host_code/sgemm_demo.c:214-242,
//   irr_*_V0.0 demos :205-222): per K block of k_block (K_G = 512): tmp = 0,
//   tmp = fma(a, b, tmp) ascending in k, c += tmp; then the tail block the
//   same way (always added); scalar beta added last;
//   three-level sum (irr_thinB_sgemm_release_V1.2/host_code/
//   irr_thinB_sgemm_demo.c:217-239): slabs of k_slab (K_A) inside blocks of
//   k_block (K_G), tmp_i += tmp_s, tmp_o += tmp_i, c = c0 + (tmp_o + beta).
// FP32 products use the double-precision fma() on float operands rounded
// back to float, as those C loops do (fma() is the double libm function).
//
// Tiling: 64x64 C tile per CTA, 256 threads, 4x4 elements per thread,
// K staged through shared memory 16 at a time.  The tiling does not change
// the per-element order.  FP64 throughput on GB300 is ~1.2 TFLOP/s, so this
// kernel is FP64-pipe bound; it is also the library's plain DGEMM.
#include "gb_common.cuh"

namespace gb {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

template <typename T>
struct Ord;

template <>
struct Ord<double> {
    __device__ static double fmac(double a, double b, double t) { return __fma_rn(a, b, t); }
    __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
};

template <>
struct Ord<float> {
    // (float) fma((double)a, (double)b, (double)t): the reference's double fma
    __device__ static float fmac(float a, float b, float t) {
        return __double2float_rn(__fma_rn((double)a, (double)b, (double)t));
    }
    __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
};

struct OrdParams {
    int64_t M, N, K, lda, ldb, ldc;
    int ta, tb;
    int64_t kg, ka;       // block and slab (ka == 0: two-level)
    int start_from_c;     // c starts from C_in (else +0)
    int scale_a, scale_b; // alpha pre-scales op(A) / op(B)
    int scalar_beta;      // add beta as a scalar at the end
    int blas_general;     // C = alpha*c + beta*C_in after the sum
};

template <typename T>
__device__ __forceinline__ void load_tiles(const T *__restrict__ A, const T *__restrict__ B, T (*As)[BM + 1],
                                           T (*Bs)[BN + 1], const OrdParams &p, int64_t m0, int64_t n0,
                                           int64_t k0, int64_t kend, T alpha) {
    const int tid = threadIdx.x;
#pragma unroll
    for (int r = 0; r < (BM * BK) / NT; r++) {
        int l = tid + r * NT;
        int mm, kk;
        if (p.ta) { mm = l % BM; kk = l / BM; } else { mm = l / BK; kk = l % BK; }
        int64_t m = m0 + mm, k = k0 + kk;
        T v = T(0);
        if (m < p.M && k < kend) v = p.ta ? A[k * p.lda + m] : A[m * p.lda + k];
        if (p.scale_a) v = Ord<T>::mul(alpha, v);
        As[kk][mm] = v;
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / NT; r++) {
        int l = tid + r * NT;
        int nn, kk;
        if (p.tb) { nn = l / BK; kk = l % BK; } else { nn = l % BN; kk = l / BN; }
        int64_t n = n0 + nn, k = k0 + kk;
        T v = T(0);
        if (n < p.N && k < kend) v = p.tb ? B[n * p.ldb + k] : B[k * p.ldb + n];
        if (p.scale_b) v = Ord<T>::mul(alpha, v);
        Bs[kk][nn] = v;
    }
}

// Sum op(A)op(B) over k in [ks, ke) into t (a fresh chain, t starts at 0).
template <typename T>
__device__ __forceinline__ void chain(const T *__restrict__ A, const T *__restrict__ B, T (*As)[BM + 1],
                                      T (*Bs)[BN + 1], const OrdParams &p, int64_t m0, int64_t n0, int64_t ks,
                                      int64_t ke, T alpha, T (&t)[4][4]) {
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) t[i][j] = T(0);
    for (int64_t k0 = ks; k0 < ke; k0 += BK) {
        __syncthreads();
        load_tiles<T>(A, B, As, Bs, p, m0, n0, k0, ke, alpha);
        __syncthreads();
        int kn = (int)((ke - k0) < BK ? (ke - k0) : BK);
        for (int kk = 0; kk < kn; kk++) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) t[i][j] = Ord<T>::fmac(a[i], b[j], t[i][j]);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(NT) gemm_ordered_kernel(const T *__restrict__ A, const T *__restrict__ B,
                                                          T *__restrict__ C, OrdParams p, T alpha, T beta) {
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;

    T c[4][4], t[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int64_t m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
            c[i][j] = (p.start_from_c && m < p.M && n < p.N) ? C[m * p.ldc + n] : T(0);
        }

    if (p.ka == 0) {
        // two-level: full K blocks, then the (possibly empty) tail block
        const int64_t kfull = p.K - p.K % p.kg;
        for (int64_t kb = 0; kb < kfull; kb += p.kg) {
            chain<T>(A, B, As, Bs, p, m0, n0, kb, kb + p.kg, alpha, t);
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) c[i][j] = Ord<T>::add(c[i][j], t[i][j]);
        }
        chain<T>(A, B, As, Bs, p, m0, n0, kfull, p.K, alpha, t);
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                c[i][j] = Ord<T>::add(c[i][j], t[i][j]);
                if (p.scalar_beta) c[i][j] = Ord<T>::add(c[i][j], beta);
            }
    } else {
        // three-level: slabs of ka inside blocks of kg (min-sized at the end)
        T to[4][4], ti[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) to[i][j] = T(0);
        for (int64_t ko = 0; ko < p.K; ko += p.kg) {
            int64_t kgc = p.kg < p.K - ko ? p.kg : p.K - ko;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) ti[i][j] = T(0);
            for (int64_t ki = 0; ki < kgc; ki += p.ka) {
                int64_t kac = p.ka < kgc - ki ? p.ka : kgc - ki;
                chain<T>(A, B, As, Bs, p, m0, n0, ko + ki, ko + ki + kac, alpha, t);
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) ti[i][j] = Ord<T>::add(ti[i][j], t[i][j]);
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) to[i][j] = Ord<T>::add(to[i][j], ti[i][j]);
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                T s = p.scalar_beta ? Ord<T>::add(to[i][j], beta) : to[i][j];
                c[i][j] = Ord<T>::add(c[i][j], s);
            }
    }

#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int64_t m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
            if (m < p.M && n < p.N) {
                T v = c[i][j];
                if (p.blas_general) {
                    T bc = (beta == T(0)) ? T(0) : Ord<T>::mul(beta, C[m * p.ldc + n]);
                    v = Ord<T>::add(Ord<T>::mul(alpha, v), bc);
                }
                C[m * p.ldc + n] = v;
            }
        }
}

template <typename T>
gb_status launch(const GemmArgs &g) {
    OrdParams p;
    p.M = g.M; p.N = g.N; p.K = g.K;
    p.lda = g.lda; p.ldb = g.ldb; p.ldc = g.ldc;
    p.ta = g.ta; p.tb = g.tb;
    p.kg = g.k_block > 0 ? g.k_block : 512;
    p.ka = g.k_slab > 0 ? g.k_slab : 0;
    p.start_from_c = 0; p.scale_a = 0; p.scale_b = 0; p.scalar_beta = 0; p.blas_general = 0;
    if (g.semantics == GB_SEM_BLAS) {
        if (g.alpha == 1.0 && g.beta == 1.0) {
            p.start_from_c = 1;                 // C += op(A)op(B), the reference update
        } else {
            p.blas_general = 1;                 // C = alpha*sum + beta*C
        }
    } else {
        p.scalar_beta = 1;
        p.start_from_c = (g.semantics == GB_SEM_ACCUM_SCALAR_BETA);
        if (g.alpha_on_b) p.scale_b = 1; else p.scale_a = 1;
    }
    if (g.M == 0 || g.N == 0) return ok();
    dim3 grid((unsigned)ceil_div(g.N, BN), (unsigned)ceil_div(g.M, BM));
    if (grid.y > 65535u) return set_status(GB_ERR_UNSUPPORTED, "ordered gemm: M too large (%lld)", (long long)g.M);
    gemm_ordered_kernel<T><<<grid, NT, 0, g.stream>>>((const T *)g.A, (const T *)g.B, (T *)g.C, p, (T)g.alpha,
                                                     (T)g.beta);
    GB_LAUNCH_CHECK("gemm_ordered_kernel");
    return ok();
}

}  // namespace

gb_status launch_gemm_ordered_f64(const GemmArgs &g) { return launch<double>(g); }
gb_status launch_gemm_ordered_f32(const GemmArgs &g) { return launch<float>(g); }

}  // namespace gb
