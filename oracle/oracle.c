/*
 * oracle.c -- CPU restatement of the reference's host-side check loops.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See oracle.h for the contract;
 * every function cites the reference loop it restates.  Build flags keep
 * the arithmetic literal: -O2 -std=c99 -ffp-contract=off (no fused
 * multiply-adds other than the explicit fma() calls the reference makes).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OFFSET(row, col, ld) ((row) * (ld) + (col))

static int g_threads = 0;

void gbo_set_threads(int n) { g_threads = n; }

int gbo_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_num_procs();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------- generator */
uint64_t gbo_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static inline uint64_t gbo_bits(uint64_t seed, uint64_t idx)
{
    return gbo_mix64(gbo_mix64(seed) + (idx + 1) * 0x9E3779B97F4A7C15ULL);
}

double gbo_unit(uint64_t seed, uint64_t idx)
{
    return (double)(gbo_bits(seed, idx) >> 11) * 0x1.0p-53;
}

static inline double gbo_value(uint64_t seed, uint64_t idx, int kind)
{
    double u = gbo_unit(seed, idx);
    if (kind == 1) return u;
    double v = 2.0 * u - 1.0;                         /* exact */
    if (kind == 2) {
        /* exponent stream: a second seed, e uniform in {-20..20} */
        int e = (int)(gbo_bits(seed ^ 0x5851F42D4C957F2DULL, idx) % 41ULL) - 20;
        v = ldexp(v, e);
    }
    return v;
}

void gbo_fill_f64(double *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) schedule(static)
    for (int64_t r = 0; r < rows; r++)
        for (int64_t c = 0; c < cols; c++)
            X[OFFSET(r, c, ld)] = gbo_value(seed, (uint64_t)(r * cols + c), kind);
}

void gbo_fill_f32(float *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) schedule(static)
    for (int64_t r = 0; r < rows; r++)
        for (int64_t c = 0; c < cols; c++)
            X[OFFSET(r, c, ld)] = (float)gbo_value(seed, (uint64_t)(r * cols + c), kind);
}

/* op(A)(i,k) and op(B)(k,j) for row-major storage */
#define OPA(i, k) (ta ? A[OFFSET((k), (i), lda)] : A[OFFSET((i), (k), lda)])
#define OPB(k, j) (tb ? B[OFFSET((j), (k), ldb)] : B[OFFSET((k), (j), ldb)])

/* ------------------------------------------------------------------ DGEMM */
/* dgemm_release_V1.1/host_code/dgemm_demo.c:233-252 */
void gbo_dgemm_ref(int ta, int tb, int64_t M, int64_t N, int64_t K,
                   const double *A, int64_t lda, const double *B, int64_t ldb,
                   double *C, int64_t ldc, int64_t kg)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++) {
        for (int64_t j = 0; j < N; j++) {
            for (int64_t k = 0; k < K - K % kg; k += kg) {
                double tmp = 0.0;
                for (int64_t kk = 0; kk < kg; kk++)
                    tmp = fma(OPA(i, k + kk), OPB(k + kk, j), tmp);
                C[OFFSET(i, j, ldc)] += tmp;
            }
            double tmp = 0.0;
            for (int64_t k = K - K % kg; k < K; k++)
                tmp = fma(OPA(i, k), OPB(k, j), tmp);
            C[OFFSET(i, j, ldc)] += tmp;
        }
    }
}

/* ------------------------------------------------------------------ SGEMM */
/* sgemm_release_V1.3.2/host_code/sgemm_demo.c:214-242.  alpha*a is a float
 * product (both operands float); fma() is the double-precision libm call,
 * its result is rounded to float on assignment to the float tmp. */
void gbo_sgemm_ref(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha,
                   const float *A, int64_t lda, const float *B, int64_t ldb,
                   float beta, float *C, int64_t ldc, int64_t kg, int accumulate)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++) {
        for (int64_t j = 0; j < N; j++) {
            float c = accumulate ? C[OFFSET(i, j, ldc)] : 0.0f;
            for (int64_t k = 0; k < K - K % kg; k += kg) {
                float tmp = 0.0f;
                for (int64_t kk = 0; kk < kg; kk++) {
                    float as = alpha * OPA(i, k + kk);
                    tmp = (float)fma((double)as, (double)OPB(k + kk, j), (double)tmp);
                }
                c += tmp;
            }
            float tmp = 0.0f;
            for (int64_t k = K - K % kg; k < K; k++) {
                float as = alpha * OPA(i, k);
                tmp = (float)fma((double)as, (double)OPB(k, j), (double)tmp);
            }
            c += tmp;
            c += beta;
            C[OFFSET(i, j, ldc)] = c;
        }
    }
}

/* irr_shortA_sgemm_release_V0.0/host_code/irr_shortA_sgemm_demo.c:206-222 */
void gbo_sgemm_irr_ref(int ta, int tb, int64_t M, int64_t N, int64_t K,
                       const float *A, int64_t lda, const float *B, int64_t ldb,
                       float *C, int64_t ldc, int64_t kg)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++) {
        for (int64_t j = 0; j < N; j++) {
            for (int64_t k = 0; k < K - K % kg; k += kg) {
                float tmp = 0.0f;
                for (int64_t kk = 0; kk < kg; kk++)
                    tmp = (float)fma((double)OPA(i, k + kk), (double)OPB(k + kk, j), (double)tmp);
                C[OFFSET(i, j, ldc)] += tmp;
            }
            float tmp = 0.0f;
            for (int64_t k = K - K % kg; k < K; k++)
                tmp = (float)fma((double)OPA(i, k), (double)OPB(k, j), (double)tmp);
            C[OFFSET(i, j, ldc)] += tmp;
        }
    }
}

/* irr_thinB_sgemm_release_V1.2/host_code/irr_thinB_sgemm_demo.c:217-239 */
void gbo_thinB_sgemm_ref(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha,
                         const float *A, int64_t lda, const float *B, int64_t ldb,
                         float beta, float *C, int64_t ldc, int64_t kg, int64_t ka,
                         int accumulate)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++) {
        for (int64_t j = 0; j < N; j++) {
            float tmp_o = 0.0f;
            for (int64_t k_o = 0; k_o < K; k_o += kg) {
                int64_t kg_cur = kg < K - k_o ? kg : K - k_o;
                float tmp_i = 0.0f;
                for (int64_t k_i = 0; k_i < kg_cur; k_i += ka) {
                    int64_t ka_cur = ka < kg_cur - k_i ? ka : kg_cur - k_i;
                    float tmp_s = 0.0f;
                    for (int64_t k_s = 0; k_s < ka_cur; k_s++) {
                        int64_t k = k_o + k_i + k_s;
                        float bs = alpha * OPB(k, j);
                        tmp_s = (float)fma((double)OPA(i, k), (double)bs, (double)tmp_s);
                    }
                    tmp_i += tmp_s;
                }
                tmp_o += tmp_i;
            }
            float c0 = accumulate ? C[OFFSET(i, j, ldc)] : 0.0f;
            C[OFFSET(i, j, ldc)] = c0 + (tmp_o + beta);
        }
    }
}

/* -------------------------------------------------------------- transpose */
/* transpose/host_code/transpose.c:113-119 */
void gbo_transpose_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++)
        for (int64_t j = 0; j < N; j++)
            memcpy(&B[OFFSET(j, i, ldb)], &A[OFFSET(i, j, lda)], sizeof(float));
}

void gbo_transpose_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++)
        for (int64_t j = 0; j < N; j++)
            memcpy(&B[OFFSET(j, i, ldb)], &A[OFFSET(i, j, lda)], sizeof(double));
}

/* Transpose-accumulate B += A^T: the semantics of the reference's
 * micro_kernel_16x16_add / micro_kernel_16x16x2_add
 * (dgemm_release_V1.1/device_code/dgemm_kernel.c:174, :635) and
 * micro_kernel_float_32x32_add (sgemm_release_V1.3.1/device_code/
 * sgemm_kernel.c:482), which add a transposed tile into C; one IEEE add per
 * element. */
void gbo_transpose_add_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++)
        for (int64_t j = 0; j < N; j++)
            B[OFFSET(j, i, ldb)] = B[OFFSET(j, i, ldb)] + A[OFFSET(i, j, lda)];
}

void gbo_transpose_add_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb)
{
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t i = 0; i < M; i++)
        for (int64_t j = 0; j < N; j++)
            B[OFFSET(j, i, ldb)] = B[OFFSET(j, i, ldb)] + A[OFFSET(i, j, lda)];
}

/* ---------------------------------------------------------------- stencil */
/* stencil_2d_V1.2/host_code/matrix_stencil.c:35-48 with a working pointer
 * swap (the reference's switch_pointer at :28-33 swaps copies) and the
 * device layout for B (padded, interior at (row+1, col+1), as
 * kernel_stencil.c:1096 writes it). */
#define STENCIL_BODY(T, FIVE)                                                   \
    int nt = gbo_get_threads();                                                 \
    const int64_t ld = N + 2;                                                   \
    for (int it = 0; it < iters; it++) {                                        \
        const T *src = (it % 2 == 0) ? A : B;                                   \
        T *dst = (it % 2 == 0) ? B : A;                                         \
        _Pragma("omp parallel for num_threads(nt) schedule(static)")            \
        for (int64_t row = 0; row < M; row++) {                                 \
            for (int64_t col = 0; col < N; col++) {                             \
                T top = src[(row) * ld + col + 1];                              \
                T left = src[(row + 1) * ld + col];                             \
                T right = src[(row + 1) * ld + col + 2];                        \
                T down = src[(row + 2) * ld + col + 1];                         \
                T middle = src[(row + 1) * ld + col + 1];                       \
                T r;                                                            \
                if (order == 0)                                                 \
                    r = (top + left + right + down + middle) * FIVE;            \
                else if (order == 1)                                            \
                    r = FIVE * (top + middle + down + left + right);            \
                else if ((row & 1) == 0)                                        \
                    r = (right + ((left + top) + (middle + down))) * FIVE;      \
                else                                                            \
                    r = (right + ((left + down) + (top + middle))) * FIVE;      \
                dst[(row + 1) * ld + col + 1] = r;                              \
            }                                                                   \
        }                                                                       \
    }

void gbo_stencil_f64(int64_t M, int64_t N, double *A, double *B, int iters, int order)
{
    STENCIL_BODY(double, 0.2)
}

void gbo_stencil_f32(int64_t M, int64_t N, float *A, float *B, int iters, int order)
{
    STENCIL_BODY(float, 0.2f)
}

/* 9-point stencil with a 3x3 weight window w (row-major: w[0..2] the row
 * above, w[3..5] the row itself, w[6..8] the row below), the generalisation
 * of stencil_2d named as the next step of the hot path.  Order: the first
 * product rounded, then eight fused multiply-adds in window order.  Same
 * padded layout and ping-pong as gbo_stencil; the halo is never written. */
#define STENCIL9_BODY(T, FMA)                                                   \
    int nt = gbo_get_threads();                                                 \
    const int64_t ld = N + 2;                                                   \
    for (int it = 0; it < iters; it++) {                                        \
        const T *src = (it % 2 == 0) ? A : B;                                   \
        T *dst = (it % 2 == 0) ? B : A;                                         \
        _Pragma("omp parallel for num_threads(nt) schedule(static)")            \
        for (int64_t row = 0; row < M; row++) {                                 \
            for (int64_t col = 0; col < N; col++) {                             \
                const T *p = src + row * ld + col;   /* window top-left */      \
                T r = w[0] * p[0];                                              \
                r = FMA(w[1], p[1], r);                                         \
                r = FMA(w[2], p[2], r);                                         \
                r = FMA(w[3], p[ld], r);                                        \
                r = FMA(w[4], p[ld + 1], r);                                    \
                r = FMA(w[5], p[ld + 2], r);                                    \
                r = FMA(w[6], p[2 * ld], r);                                    \
                r = FMA(w[7], p[2 * ld + 1], r);                                \
                r = FMA(w[8], p[2 * ld + 2], r);                                \
                dst[(row + 1) * ld + col + 1] = r;                              \
            }                                                                   \
        }                                                                       \
    }

void gbo_stencil9_f64(int64_t M, int64_t N, double *A, double *B, int iters, const double *w)
{
    STENCIL9_BODY(double, fma)
}

void gbo_stencil9_f32(int64_t M, int64_t N, float *A, float *B, int iters, const float *w)
{
    STENCIL9_BODY(float, fmaf)
}

/* -------------------------------------------------------- accuracy oracle */
/* Error-free transformations (Ogita, Rump & Oishi 2005). */
static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b;
    double z = x - a;
    *e = (a - (x - z)) + (b - z);
    *s = x;
}

static inline void two_prod(double a, double b, double *p, double *e)
{
    double x = a * b;
    *e = fma(a, b, -x);
    *p = x;
}

/* alpha * sum_k x_k y_k + beta * c, each term added with TwoSum into (p, s) */
#define DOT2_BODY(XK, YK)                                                       \
    double p = 0.0, s = 0.0;                                                    \
    for (int64_t k = 0; k < K; k++) {                                           \
        double h, r, q;                                                         \
        two_prod((double)(XK), (double)(YK), &h, &r);                           \
        two_sum(p, h, &p, &q);                                                  \
        s += q + r;                                                             \
    }                                                                           \
    double ph, pe, sh, out_p, q1, q2, bh, be;                                   \
    two_prod(alpha, p, &ph, &pe);                                               \
    two_prod(beta, c0, &bh, &be);                                               \
    two_sum(ph, bh, &out_p, &q1);                                               \
    sh = alpha * s;                                                             \
    q2 = (q1 + pe) + (be + sh);                                                 \
    Cref[a * nc + b] = out_p + q2;

void gbo_gemm_dot2_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha,
                       const double *A, int64_t lda, const double *B, int64_t ldb,
                       double beta, const double *C0, int64_t ldc,
                       const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                       double *Cref)
{
    (void)M; (void)N;
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t a = 0; a < nr; a++) {
        for (int64_t b = 0; b < nc; b++) {
            int64_t i = rows[a], j = cols[b];
            double c0 = (C0 && beta != 0.0) ? C0[OFFSET(i, j, ldc)] : 0.0;
            DOT2_BODY(OPA(i, k), OPB(k, j))
        }
    }
}

void gbo_gemm_dot2_f32(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha,
                       const float *A, int64_t lda, const float *B, int64_t ldb,
                       double beta, const float *C0, int64_t ldc,
                       const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                       double *Cref)
{
    (void)M; (void)N;
    int nt = gbo_get_threads();
    #pragma omp parallel for num_threads(nt) collapse(2) schedule(static)
    for (int64_t a = 0; a < nr; a++) {
        for (int64_t b = 0; b < nc; b++) {
            int64_t i = rows[a], j = cols[b];
            double c0 = (C0 && beta != 0.0) ? (double)C0[OFFSET(i, j, ldc)] : 0.0;
            DOT2_BODY(OPA(i, k), OPB(k, j))
        }
    }
}

#define NORMS_BODY                                                              \
    int nt = gbo_get_threads();                                                 \
    _Pragma("omp parallel for num_threads(nt) schedule(static)")                \
    for (int64_t a = 0; a < nr; a++) {                                          \
        double s = 0.0;                                                         \
        for (int64_t k = 0; k < K; k++) { double v = OPA(rows[a], k); s += v * v; } \
        rn2[a] = s;                                                             \
    }                                                                           \
    _Pragma("omp parallel for num_threads(nt) schedule(static)")                \
    for (int64_t b = 0; b < nc; b++) {                                          \
        double s = 0.0;                                                         \
        for (int64_t k = 0; k < K; k++) { double v = OPB(k, cols[b]); s += v * v; } \
        cn2[b] = s;                                                             \
    }

void gbo_op_norms_f64(int ta, int tb, int64_t M, int64_t N, int64_t K,
                      const double *A, int64_t lda, const double *B, int64_t ldb,
                      const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                      double *rn2, double *cn2)
{
    (void)M; (void)N;
    NORMS_BODY
}

void gbo_op_norms_f32(int ta, int tb, int64_t M, int64_t N, int64_t K,
                      const float *A, int64_t lda, const float *B, int64_t ldb,
                      const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                      double *rn2, double *cn2)
{
    (void)M; (void)N;
    NORMS_BODY
}
