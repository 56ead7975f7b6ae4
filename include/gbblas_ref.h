/*
 * gbblas_ref.h -- the reference's own device entry points, by name and
 * argument list, as host-callable functions backed by the GB300 kernels.
 *
 * Each declaration cites the reference header it replaces (paths relative to
 * the VVinstonSmith/BLAS-for-multi-core-DSP root).  Argument order and
 * meaning are the reference's; "unlong" is unsigned long as there.  Barrier
 * ids (b_id, bid_main, bid_T) are accepted and ignored: there are no DSP
 * barriers on the GPU.  Pointers are device pointers.  The functions return
 * void as the reference's do; the status of the call is recorded for
 * gb_get_last_status() / gb_last_error() (gbblas.h).
 *
 * They run on the stream set by gb_ref_set_stream (default: the legacy
 * default stream) and are asynchronous: call gb_sync() before reading C on
 * the host, as the reference host calls hthread_group_wait().
 *
 * Arithmetic: by default the GEMMs use GB_ALGO_ORDERED, which reproduces
 * the reference's host check loop bit for bit (K blocks of 512, alpha
 * placement, float/double rounding); gb_ref_set_algo() selects a fast
 * algorithm instead (results then match within the normwise bound).
 *
 * Names shared by several reference packages with different argument lists
 * exist once: transpose_A2B is the ld-aware DGEMM V1.1 one
 * (dgemm_release_V1.1/include/dgemm_kernel.h:36), irr_thinB_sgemm_* are the
 * V1.2 ones (with alpha, beta), sgemm_*_qxx are the V1.3.2 ones.
 */
#ifndef GBBLAS_REF_H
#define GBBLAS_REF_H

#include "gbblas.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef unlong
#define unlong unsigned long
#endif

void gb_ref_set_stream(void *stream);
void gb_ref_set_algo(int algo);   /* gb_algo; GB_ALGO_ORDERED by default */

/* dgemm_release_V1.1/include/dgemm_kernel.h:36-67 -- C += op(A)op(B),
 * A0 (rows x lda), B0 (rows x ldb), C0 (M x ldc) */
void transpose_A2B(unlong lda, unlong ldb, unlong M, unlong N, unlong b_id, double *A, double *B);
void dgemm_NN(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);
void dgemm_NT(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);
void dgemm_TN(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C);
void dgemm_TT(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);
void dgemm_null(unlong lda, unlong ldb, unlong ldc, unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);

/* sgemm_release_V1.3.2/include/sgemm_kernel.h:8-26 -- C = alpha*op(A)op(B) + beta
 * (beta a scalar; no leading dimensions: lda = K or M, ldb = N or K, ldc = N) */
void transpose_A2B_float32(unlong M, unlong N, unlong b_id, float *A, float *B);
void sgemm_NN_qxx(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta);
void sgemm_NT_qxx(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta);
void sgemm_TN_qxx(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C, float alpha, float beta);
void sgemm_TT_qxx(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta);
void sgemm_null(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta);

/* irr_shortA_sgemm_release_V0.0/include/irr_shortA_sgemm_kernel.h:11-26 -- C += op(A)op(B) */
void irr_shortA_sgemm_NN(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C);
void irr_shortA_sgemm_NT(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C);
void irr_shortA_sgemm_TN(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C);
void irr_shortA_sgemm_TT(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C);
void irr_shortA_sgemm_null(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C);

/* irr_shortA_dgemm_release_V0.0/include/irr_shortA_dgemm_kernel.h:11-26 -- C += op(A)op(B) */
void irr_shortA_dgemm_NN_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);
void irr_shortA_dgemm_NT_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);
void irr_shortA_dgemm_TN_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C);
void irr_shortA_dgemm_TT_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C);
void irr_shortA_dgemm_null(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);

/* irr_thinB_dgemm_release_V0.0/include/irr_thinB_dgemm_kernel.h:11-26 -- C += op(A)op(B) */
void irr_thinB_dgemm_TT_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);
void irr_thinB_dgemm_NT_dbuf(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);
void irr_thinB_dgemm_TN_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C);
void irr_thinB_dgemm_NN_dbuf(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, double *A, double *B, double *C);
void irr_thinB_dgemm_null(unlong M, unlong N, unlong K, unlong b_id, double *A, double *B, double *C);

/* irr_thinB_sgemm_release_V1.2/include/irr_thinB_sgemm_kernel.h:11-26 --
 * C = alpha*op(A)op(B) + beta (scalar), three-level K sum (K_G 3072, K_A 512) */
void irr_thinB_sgemm_TT(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta);
void irr_thinB_sgemm_NT(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta);
void irr_thinB_sgemm_TN(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C, float alpha, float beta);
void irr_thinB_sgemm_NN(unlong M, unlong N, unlong K, unlong bid_main, unlong bid_T, float *A, float *B, float *C, float alpha, float beta);
void irr_thinB_sgemm_null(unlong M, unlong N, unlong K, unlong b_id, float *A, float *B, float *C, float alpha, float beta);

/* transpose/device_code/kernel.c:1167,1280,2002,2110 -- B (N x M) = A^T, A is M x N */
void transpose_16x16_dbuf(unlong M, unlong N, unlong b_id, double *A, double *B);
void transpose_null(unlong M, unlong N, unlong b_id, double *A, double *B);
void transpose_float_32x32_dbuf(unlong M, unlong N, unlong b_id, float *A, float *B);
void transpose_float_null(unlong M, unlong N, unlong b_id, float *A, float *B);

/* stencil_2d_V1.2/device_code/kernel_stencil.c:14,1042,1114 -- one Jacobi sweep
 * A -> B on (M+2) x (N+2) padded grids (row stride N+2) */
void stencil_vector(unlong M, unlong N, double *A, double *B);
void stencil_scalar(unlong M, unlong N, double *A, double *B);
void stencil_null(unlong M, unlong N, double *A, double *B);

#ifdef __cplusplus
}
#endif
#endif
