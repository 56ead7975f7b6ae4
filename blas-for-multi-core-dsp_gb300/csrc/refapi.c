/*
 * refapi.c -- the reference's device entry points by name (gbblas_ref.h)
 * and the launch-by-name boundary gb_exec (gbblas.h), in C over the
 * library's C ABI.
 *
 * Argument lists follow the reference headers cited in gbblas_ref.h; the
 * fixed alpha = 5, beta = 3 of the SGEMM launchers are the launcher globals
 * of sgemm_release_V1.3.2/device_code/sgemm_launcher.c:11-12 and
 * irr_thinB_sgemm_release_V1.2/device_code/irr_thinB_sgemm_launcher.c:11-12.
 */
#include <string.h>

#include "gbblas.h"
#include "gbblas_ref.h"

static void *g_ref_stream = NULL;
static int g_ref_algo = GB_ALGO_ORDERED;

void gb_ref_set_stream(void *stream) { g_ref_stream = stream; }
void gb_ref_set_algo(int algo) { g_ref_algo = algo; }

static gb_gemm_opts ref_opts(int semantics, int k_block, int k_slab, int alpha_on_b)
{
    gb_gemm_opts o;
    gb_gemm_opts_init(&o);
    o.stream = g_ref_stream;
    o.algo = g_ref_algo;
    o.semantics = semantics;
    o.k_block = k_block;
    o.k_slab = k_slab;
    o.alpha_on_b = alpha_on_b;
    return o;
}

/* ---------------------------------------------- dgemm_release_V1.1 */
static void dgemm_ref(char ta, char tb, unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K,
                      double *A, double *B, double *C)
{
    gb_gemm_opts o = ref_opts(GB_SEM_BLAS, 512, 0, 0);
    gb_dgemm(ta, tb, (int64_t)M, (int64_t)N, (int64_t)K, 1.0, A, (int64_t)lda, B, (int64_t)ldb, 1.0, C,
             (int64_t)ldc, &o);
}

void transpose_A2B(unlong lda, unlong ldb, unlong M, unlong N, unlong b_id, double *A, double *B)
{
    (void)b_id;
    gb_transpose_f64((int64_t)M, (int64_t)N, A, (int64_t)lda, B, (int64_t)ldb, g_ref_stream);
}
void dgemm_NN(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)b_id; dgemm_ref('N', 'N', lda, ldb, ldc, M, N, K, A, B, C); }
void dgemm_NT(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)b_id; dgemm_ref('N', 'T', lda, ldb, ldc, M, N, K, A, B, C); }
void dgemm_TN(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C)
{ (void)bid_main; (void)bid_T; dgemm_ref('T', 'N', lda, ldb, ldc, M, N, K, A, B, C); }
void dgemm_TT(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)b_id; dgemm_ref('T', 'T', lda, ldb, ldc, M, N, K, A, B, C); }
void dgemm_null(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)lda; (void)ldb; (void)ldc; (void)M; (void)N; (void)K; (void)b_id; (void)A; (void)B; (void)C; }

/* ---------------------------------------------- sgemm_release_V1.3.2 */
static void sgemm_ref(char ta, char tb, unlong M, unlong N, unlong K, float *A, float *B, float *C, float alpha,
                      float beta)
{
    gb_gemm_opts o = ref_opts(GB_SEM_SCALAR_BETA, 512, 0, 0);
    int64_t lda = ta == 'N' ? (int64_t)K : (int64_t)M, ldb = tb == 'N' ? (int64_t)N : (int64_t)K;
    gb_sgemm(ta, tb, (int64_t)M, (int64_t)N, (int64_t)K, alpha, A, lda, B, ldb, beta, C, (int64_t)N, &o);
}

void transpose_A2B_float32(unlong M, unlong N, unlong b_id, float *A, float *B)
{
    (void)b_id;
    gb_transpose_f32((int64_t)M, (int64_t)N, A, (int64_t)N, B, (int64_t)M, g_ref_stream);
}
void sgemm_NN_qxx(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta)
{ (void)b_id; sgemm_ref('N', 'N', M, N, K, A, B, C, alpha, beta); }
void sgemm_NT_qxx(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta)
{ (void)b_id; sgemm_ref('N', 'T', M, N, K, A, B, C, alpha, beta); }
void sgemm_TN_qxx(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C, float alpha, float beta)
{ (void)bid_main; (void)bid_T; sgemm_ref('T', 'N', M, N, K, A, B, C, alpha, beta); }
void sgemm_TT_qxx(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta)
{ (void)b_id; sgemm_ref('T', 'T', M, N, K, A, B, C, alpha, beta); }
void sgemm_null(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta)
{ (void)M; (void)N; (void)K; (void)b_id; (void)A; (void)B; (void)C; (void)alpha; (void)beta; }

/* ------------------------------------- irregular V0.0: C += op(A)op(B) */
static void irr_s(char ta, char tb, unlong M, unlong N, unlong K, float *A, float *B, float *C)
{
    gb_gemm_opts o = ref_opts(GB_SEM_BLAS, 512, 0, 0);
    int64_t lda = ta == 'N' ? (int64_t)K : (int64_t)M, ldb = tb == 'N' ? (int64_t)N : (int64_t)K;
    gb_sgemm(ta, tb, (int64_t)M, (int64_t)N, (int64_t)K, 1.0f, A, lda, B, ldb, 1.0f, C, (int64_t)N, &o);
}
static void irr_d(char ta, char tb, unlong M, unlong N, unlong K, double *A, double *B, double *C)
{
    gb_gemm_opts o = ref_opts(GB_SEM_BLAS, 512, 0, 0);
    int64_t lda = ta == 'N' ? (int64_t)K : (int64_t)M, ldb = tb == 'N' ? (int64_t)N : (int64_t)K;
    gb_dgemm(ta, tb, (int64_t)M, (int64_t)N, (int64_t)K, 1.0, A, lda, B, ldb, 1.0, C, (int64_t)N, &o);
}

void irr_shortA_sgemm_NN(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C)
{ (void)b_id; irr_s('N', 'N', M, N, K, A, B, C); }
void irr_shortA_sgemm_NT(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C)
{ (void)b_id; irr_s('N', 'T', M, N, K, A, B, C); }
void irr_shortA_sgemm_TN(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C)
{ (void)bid_main; (void)bid_T; irr_s('T', 'N', M, N, K, A, B, C); }
void irr_shortA_sgemm_TT(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C)
{ (void)bid_main; (void)bid_T; irr_s('T', 'T', M, N, K, A, B, C); }
void irr_shortA_sgemm_null(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C)
{ (void)M; (void)N; (void)K; (void)b_id; (void)A; (void)B; (void)C; }

void irr_shortA_dgemm_NN_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)b_id; irr_d('N', 'N', M, N, K, A, B, C); }
void irr_shortA_dgemm_NT_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)b_id; irr_d('N', 'T', M, N, K, A, B, C); }
void irr_shortA_dgemm_TN_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C)
{ (void)bid_main; (void)bid_T; irr_d('T', 'N', M, N, K, A, B, C); }
void irr_shortA_dgemm_TT_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C)
{ (void)bid_main; (void)bid_T; irr_d('T', 'T', M, N, K, A, B, C); }
void irr_shortA_dgemm_null(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)M; (void)N; (void)K; (void)b_id; (void)A; (void)B; (void)C; }

void irr_thinB_dgemm_TT_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)b_id; irr_d('T', 'T', M, N, K, A, B, C); }
void irr_thinB_dgemm_NT_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)b_id; irr_d('N', 'T', M, N, K, A, B, C); }
void irr_thinB_dgemm_TN_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C)
{ (void)bid_main; (void)bid_T; irr_d('T', 'N', M, N, K, A, B, C); }
void irr_thinB_dgemm_NN_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C)
{ (void)bid_main; (void)bid_T; irr_d('N', 'N', M, N, K, A, B, C); }
void irr_thinB_dgemm_null(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C)
{ (void)M; (void)N; (void)K; (void)b_id; (void)A; (void)B; (void)C; }

/* ------------------ irr_thinB_sgemm V1.2: C = alpha*op(A)op(B) + beta */
static void thinB_s(char ta, char tb, unlong M, unlong N, unlong K, float *A, float *B, float *C, float alpha,
                    float beta)
{
    gb_gemm_opts o = ref_opts(GB_SEM_SCALAR_BETA, 3072, 512, 1);
    int64_t lda = ta == 'N' ? (int64_t)K : (int64_t)M, ldb = tb == 'N' ? (int64_t)N : (int64_t)K;
    gb_sgemm(ta, tb, (int64_t)M, (int64_t)N, (int64_t)K, alpha, A, lda, B, ldb, beta, C, (int64_t)N, &o);
}
void irr_thinB_sgemm_TT(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta)
{ (void)b_id; thinB_s('T', 'T', M, N, K, A, B, C, alpha, beta); }
void irr_thinB_sgemm_NT(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta)
{ (void)b_id; thinB_s('N', 'T', M, N, K, A, B, C, alpha, beta); }
void irr_thinB_sgemm_TN(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C, float alpha, float beta)
{ (void)bid_main; (void)bid_T; thinB_s('T', 'N', M, N, K, A, B, C, alpha, beta); }
void irr_thinB_sgemm_NN(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C, float alpha, float beta)
{ (void)bid_main; (void)bid_T; thinB_s('N', 'N', M, N, K, A, B, C, alpha, beta); }
void irr_thinB_sgemm_null(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta)
{ (void)M; (void)N; (void)K; (void)b_id; (void)A; (void)B; (void)C; (void)alpha; (void)beta; }

/* ------------------------------------------------------- transpose */
void transpose_16x16_dbuf(unlong M, unlong N, unlong b_id, double *A, double *B)
{ (void)b_id; gb_transpose_f64((int64_t)M, (int64_t)N, A, (int64_t)N, B, (int64_t)M, g_ref_stream); }
void transpose_null(unlong M, unlong N, unlong b_id, double *A, double *B)
{ (void)M; (void)N; (void)b_id; (void)A; (void)B; }
void transpose_float_32x32_dbuf(unlong M, unlong N, unlong b_id, float *A, float *B)
{ (void)b_id; gb_transpose_f32((int64_t)M, (int64_t)N, A, (int64_t)N, B, (int64_t)M, g_ref_stream); }
void transpose_float_null(unlong M, unlong N, unlong b_id, float *A, float *B)
{ (void)M; (void)N; (void)b_id; (void)A; (void)B; }

/* ---------------------------------------------------------- stencil */
void stencil_vector(unlong M, unlong N, double *A, double *B)
{ gb_stencil2d_f64((int64_t)M, (int64_t)N, A, B, 1, GB_STENCIL_VECTOR, g_ref_stream); }
void stencil_scalar(unlong M, unlong N, double *A, double *B)
{ gb_stencil2d_f64((int64_t)M, (int64_t)N, A, B, 1, GB_STENCIL_SCALAR, g_ref_stream); }
void stencil_null(unlong M, unlong N, double *A, double *B)
{ (void)M; (void)N; (void)A; (void)B; }

/* ----------------------------------------------------- launch by name */
static int mode_of(const char *name, char *ta, char *tb)
{
    size_t L = strlen(name);
    if (L < 2) return -1;
    char a = name[L - 2], b = name[L - 1];
    if ((a != 'N' && a != 'T') || (b != 'N' && b != 'T')) return -1;
    *ta = a; *tb = b;
    return 0;
}

static gb_status bad_args(const char *name, int want_s, int want_p, int n_scalar, int n_ptr)
{
    (void)name; (void)want_s; (void)want_p; (void)n_scalar; (void)n_ptr;
    return GB_ERR_INVALID_ARG;
}

gb_status gb_exec(const char *name, int n_scalar, int n_ptr, const unsigned long *a)
{
    char ta = 'N', tb = 'N';
    if (!name || !a) return GB_ERR_INVALID_ARG;
    gb_clear_last_status();
    if (strstr(name, "null")) return GB_OK;
    if (n_ptr != 2 && n_ptr != 3) return bad_args(name, 0, 3, n_scalar, n_ptr);
    const unsigned long *p = a + n_scalar;

    if (!strncmp(name, "launch_dgemm_", 13)) {
        if (mode_of(name, &ta, &tb) || n_ptr != 3) return GB_ERR_INVALID_ARG;
        int want = (ta == 'T' && tb == 'N') ? 8 : 7;
        if (n_scalar != want) return GB_ERR_INVALID_ARG;
        dgemm_ref(ta, tb, a[0], a[1], a[2], a[3], a[4], a[5], (double *)p[0], (double *)p[1], (double *)p[2]);
    } else if (!strncmp(name, "launch_sgemm_", 13)) {
        if (mode_of(name, &ta, &tb) || n_ptr != 3) return GB_ERR_INVALID_ARG;
        int want = (ta == 'T' && tb == 'N') ? 5 : 4;
        if (n_scalar != want) return GB_ERR_INVALID_ARG;
        sgemm_ref(ta, tb, a[0], a[1], a[2], (float *)p[0], (float *)p[1], (float *)p[2], 5.0f, 3.0f);
    } else if (!strncmp(name, "launch_irr_", 11)) {
        if (mode_of(name, &ta, &tb) || n_ptr != 3 || n_scalar < 4 || n_scalar > 5) return GB_ERR_INVALID_ARG;
        if (strstr(name, "thinB_sgemm"))
            thinB_s(ta, tb, a[0], a[1], a[2], (float *)p[0], (float *)p[1], (float *)p[2], 5.0f, 3.0f);
        else if (strstr(name, "sgemm"))
            irr_s(ta, tb, a[0], a[1], a[2], (float *)p[0], (float *)p[1], (float *)p[2]);
        else if (strstr(name, "dgemm"))
            irr_d(ta, tb, a[0], a[1], a[2], (double *)p[0], (double *)p[1], (double *)p[2]);
        else
            return GB_ERR_INVALID_ARG;
    } else if (!strcmp(name, "transpose_float_32x32_dbuf")) {
        if (n_scalar != 3 || n_ptr != 2) return GB_ERR_INVALID_ARG;
        transpose_float_32x32_dbuf(a[0], a[1], a[2], (float *)p[0], (float *)p[1]);
    } else if (!strcmp(name, "transpose_16x16_dbuf")) {
        if (n_scalar != 3 || n_ptr != 2) return GB_ERR_INVALID_ARG;
        transpose_16x16_dbuf(a[0], a[1], a[2], (double *)p[0], (double *)p[1]);
    } else if (!strcmp(name, "stencil_vector") || !strcmp(name, "stencil_scalar")) {
        if (n_scalar != 2 || n_ptr != 2) return GB_ERR_INVALID_ARG;
        gb_stencil2d_f64((int64_t)a[0], (int64_t)a[1], (double *)p[0], (double *)p[1], 1,
                         name[8] == 'v' ? GB_STENCIL_VECTOR : GB_STENCIL_SCALAR, g_ref_stream);
    } else {
        return GB_ERR_INVALID_ARG;
    }
    int st = gb_get_last_status();
    if (st != GB_OK) return (gb_status)st;
    return gb_sync(g_ref_stream);
}
