/*
 * oracle.h -- CPU restatement of the reference's host-side check loops.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * library (libgbblas): only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.  The
 * product path never links or calls it.
 *
 * Every function states the reference file:line whose arithmetic it
 * restates.  Paths are relative to the VVinstonSmith/BLAS-for-multi-core-DSP
 * project root.  The arithmetic (operand order, fma vs mul+add, K blocking,
 * float vs double intermediates) is kept exactly as in those loops, so the
 * results are bit-identical to what the reference's own check computes.
 *
 * Layout convention (the reference's): row-major, OFFSET(r,c,ld) = r*ld+c.
 * A transposed operand is stored transposed: op(A)=A^T means the buffer is
 * K x M with leading dimension lda >= M.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- inputs */
/* Counter-based generator shared bit-for-bit by the oracle, the CUDA
 * library (gb_fill_*) and numpy (tests): SplitMix64 finaliser of
 * mix(seed) + (idx+1)*0x9E3779B97F4A7C15. */
uint64_t gbo_mix64(uint64_t z);
double   gbo_unit(uint64_t seed, uint64_t idx);      /* [0,1), 53-bit grid   */
/* Fill a rows x cols row-major matrix (leading dimension ld).  Element
 * (r,c) gets value f(seed, r*cols+c), independent of ld.
 * kind 0: U[-1,1]   kind 1: U[0,1]   kind 2: ldexp(U[-1,1], e), e~U{-20..20} */
void gbo_fill_f64(double *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind);
void gbo_fill_f32(float *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind);

/* ----------------------------------------------------------------- GEMM */
/* ta/tb: 0 = 'N', 1 = 'T'.  kg = K-block length (reference K_G). */

/* dgemm_release_V1.1/host_code/dgemm_demo.c:233-252 (also the V0.0
 * irregular DGEMM demos, irr_shortA_dgemm_demo.c:205-221,
 * irr_thinB_dgemm_demo.c:205-221): C += op(A)op(B), per element: for each
 * full K block tmp=0; tmp=fma(a,b,tmp) ascending; C+=tmp; then the tail
 * block the same way (always added, even when empty). */
void gbo_dgemm_ref(int ta, int tb, int64_t M, int64_t N, int64_t K,
                   const double *A, int64_t lda, const double *B, int64_t ldb,
                   double *C, int64_t ldc, int64_t kg);

/* sgemm_release_V1.3.2/host_code/sgemm_demo.c:214-242 (V1.3.1 identical,
 * sgemm_release_V1.3.1/host_code/sgemm_demo.c:214-242):
 * tmp = (float) fma((double)(alpha*a), (double)b, (double)tmp)  -- the
 * double-precision fma() on float operands, rounded back to float --
 * C += tmp per K block, then C += beta (a scalar).
 * accumulate=0: C starts from +0.0 (V1.3.2 overwrite semantics, the
 * demo's memset C_cpu); accumulate=1: C starts from its input (V1.3.1). */
void gbo_sgemm_ref(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha,
                   const float *A, int64_t lda, const float *B, int64_t ldb,
                   float beta, float *C, int64_t ldc, int64_t kg, int accumulate);

/* irr_shortA_sgemm_release_V0.0/host_code/irr_shortA_sgemm_demo.c:206-222
 * (and irr_thinB_sgemm_release_V0.0, same loop): C += op(A)op(B) in float
 * with the double fma() rounded back to float, K blocks of kg. */
void gbo_sgemm_irr_ref(int ta, int tb, int64_t M, int64_t N, int64_t K,
                       const float *A, int64_t lda, const float *B, int64_t ldb,
                       float *C, int64_t ldc, int64_t kg);

/* irr_thinB_sgemm_release_V1.2/host_code/irr_thinB_sgemm_demo.c:217-239:
 * three-level sum, tmp_s = fma(a, alpha*b, tmp_s) over K_A slabs inside K_G
 * blocks; tmp_i += tmp_s; tmp_o += tmp_i; C = c0 + (tmp_o + beta).
 * The device kernel overwrites C (the demo seeds the device C with 999 at
 * :84 and checks against a C_cpu that started at 0), so accumulate=0
 * starts c0 from +0.0; accumulate=1 starts from the input C. */
void gbo_thinB_sgemm_ref(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha,
                         const float *A, int64_t lda, const float *B, int64_t ldb,
                         float beta, float *C, int64_t ldc, int64_t kg, int64_t ka,
                         int accumulate);

/* -------------------------------------------------------------- transpose */
/* transpose/host_code/transpose.c:113-119: B[j][i] = A[i][j], A is M x N
 * (lda >= N), B is N x M (ldb >= M).  The device kernel
 * (transpose/device_code/kernel.c:2002) is a DMA copy, so the restatement
 * copies bits. */
void gbo_transpose_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb);
void gbo_transpose_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb);
/* 9-point stencil, 3x3 weight window, first product then 8 fmas */
void gbo_stencil9_f64(int64_t M, int64_t N, double *A, double *B, int iters, const double *w);
void gbo_stencil9_f32(int64_t M, int64_t N, float *A, float *B, int iters, const float *w);
/* B += A^T (transpose-accumulate of the reference's *_add micro-kernels) */
void gbo_transpose_add_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb);
void gbo_transpose_add_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb);

/* --------------------------------------------------------------- stencil */
/* One 5-point Jacobi sweep per iteration on an (M+2)x(N+2) padded grid,
 * ping-ponging A and B; the halo is never written.  The result of `iters`
 * sweeps ends in B when iters is odd, in A when it is even.
 * order 0 (host):   ((((top+left)+right)+down)+middle)*0.2
 *                    stencil_2d_V1.2/host_code/matrix_stencil.c:40-45
 * order 1 (scalar): 0.2*((((top+middle)+down)+left)+right)
 *                    stencil_2d_V1.2/device_code/kernel_stencil.c:70-75
 * order 2 (vector V3): even interior rows right+((left+top)+(middle+down)),
 *                    odd rows right+((left+down)+(top+middle)), then *0.2
 *                    stencil_2d_V1.2/readme.txt:203-263
 * The FP32 variant (new; the reference is FP64 only) uses 0.2f. */
void gbo_stencil_f64(int64_t M, int64_t N, double *A, double *B, int iters, int order);
void gbo_stencil_f32(int64_t M, int64_t N, float *A, float *B, int iters, int order);

/* -------------------------------------------------------- accuracy oracle */
/* Reference values alpha*op(A)op(B) + beta*C0 for the rows/cols listed,
 * each dot product by Dot2 (Ogita, Rump & Oishi, SIAM J. Sci. Comput. 26(6),
 * 2005, Algorithm 5.3: TwoProduct via fma + TwoSum), i.e. as if computed in
 * twice the working precision.  Cref is nr x nc (row-major, dense). */
void gbo_gemm_dot2_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha,
                       const double *A, int64_t lda, const double *B, int64_t ldb,
                       double beta, const double *C0, int64_t ldc,
                       const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                       double *Cref);
void gbo_gemm_dot2_f32(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha,
                       const float *A, int64_t lda, const float *B, int64_t ldb,
                       double beta, const float *C0, int64_t ldc,
                       const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                       double *Cref);
/* Row norms ||op(A)(i,:)||_2^2 and column norms ||op(B)(:,j)||_2^2 for the
 * listed rows/cols (denominator of the normwise error). */
void gbo_op_norms_f64(int ta, int tb, int64_t M, int64_t N, int64_t K,
                      const double *A, int64_t lda, const double *B, int64_t ldb,
                      const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                      double *rn2, double *cn2);
void gbo_op_norms_f32(int ta, int tb, int64_t M, int64_t N, int64_t K,
                      const float *A, int64_t lda, const float *B, int64_t ldb,
                      const int64_t *rows, int64_t nr, const int64_t *cols, int64_t nc,
                      double *rn2, double *cn2);

/* Threads used by the OpenMP loops above (0 = all host cores). */
void gbo_set_threads(int n);
int  gbo_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
