/*
 * hthread_demo.c -- a host program written against the reference's host
 * runtime interface (hthread_host.h), linked with libgbblas: device buffers
 * from hthread_malloc, kernels run by name through hthread_group_exec with
 * scalars-then-pointers packing, hthread_group_wait, then a CPU check.
 * Integration test of the hthread shim (TEST INFRASTRUCTURE).
 *
 * Checks, bit for bit: launch_dgemm_{NN,NT,TN,TT} (C += op(A)op(B) with
 * K blocks of 512, the reference order), launch_sgemm_NN (C = 5*AB + 3), and
 * transpose_float_32x32_dbuf.  Prints "Success!" per check; exit 0 if all pass.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "hthread_host.h"

#define OFFSET(row, col, ld) ((row) * (ld) + (col))

static double val(long i) { return (double)((i * 2654435761u) % 1000) / 500.0 - 1.0; }

int main(void)
{
    const long M = 70, N = 90, K = 1100, K_G = 512;
    int fails = 0;
    hthread_dev_open(0);
    hthread_dat_load(0, "gbblas");
    double *A = hthread_malloc(0, M * K * sizeof(double), HT_MEM_RO);
    double *A_T = hthread_malloc(0, M * K * sizeof(double), HT_MEM_RO);
    double *B = hthread_malloc(0, K * N * sizeof(double), HT_MEM_RO);
    double *B_T = hthread_malloc(0, K * N * sizeof(double), HT_MEM_RO);
    double *C[4], *C_cpu = calloc(M * N, sizeof(double));
    for (int m = 0; m < 4; m++) C[m] = hthread_malloc(0, M * N * sizeof(double), HT_MEM_WO);
    for (long i = 0; i < M; i++)
        for (long k = 0; k < K; k++) A[OFFSET(i, k, K)] = A_T[OFFSET(k, i, M)] = val(i * K + k);
    for (long k = 0; k < K; k++)
        for (long j = 0; j < N; j++) B[OFFSET(k, j, N)] = B_T[OFFSET(j, k, K)] = val(7 + k * N + j);
    for (int m = 0; m < 4; m++)
        for (long i = 0; i < M * N; i++) C[m][i] = 0.0;

    int bid = hthread_barrier_create(0), bid_T = hthread_barrier_create(0);
    int tg = hthread_group_create(0, 8);
    const char *names[4] = {"launch_dgemm_NN", "launch_dgemm_NT", "launch_dgemm_TN", "launch_dgemm_TT"};
    for (int m = 0; m < 4; m++) {
        int ta = m >= 2, tb = m % 2;
        unsigned long args[11];
        int ns = 0;
        args[ns++] = ta ? M : K; args[ns++] = tb ? K : N; args[ns++] = N;
        args[ns++] = M; args[ns++] = N; args[ns++] = K; args[ns++] = bid;
        if (m == 2) args[ns++] = bid_T;
        args[ns] = (unsigned long)(ta ? A_T : A);
        args[ns + 1] = (unsigned long)(tb ? B_T : B);
        args[ns + 2] = (unsigned long)C[m];
        if (hthread_group_exec(tg, names[m], ns, 3, args) != 0) { printf("exec %s failed\n", names[m]); return 2; }
        hthread_group_wait(tg);
    }
    /* dgemm_demo.c's check loop */
    for (long i = 0; i < M; i++)
        for (long j = 0; j < N; j++) {
            for (long k = 0; k < K - K % K_G; k += K_G) {
                double tmp = 0.0;
                for (long kk = 0; kk < K_G; kk++) tmp = fma(A[OFFSET(i, k + kk, K)], B[OFFSET(k + kk, j, N)], tmp);
                C_cpu[OFFSET(i, j, N)] += tmp;
            }
            double tmp = 0.0;
            for (long k = K - K % K_G; k < K; k++) tmp = fma(A[OFFSET(i, k, K)], B[OFFSET(k, j, N)], tmp);
            C_cpu[OFFSET(i, j, N)] += tmp;
        }
    for (int m = 0; m < 4; m++) {
        long bad = 0;
        for (long i = 0; i < M * N; i++) bad += C[m][i] != C_cpu[i];
        printf("%s: %s (%ld mismatches)\n", names[m], bad ? "Result Error!" : "Success!", bad);
        fails += bad != 0;
    }

    /* sgemm V1.3.2 NN through the launcher packing (alpha = 5, beta = 3) */
    float *fA = hthread_malloc(0, M * K * sizeof(float), HT_MEM_RO);
    float *fB = hthread_malloc(0, K * N * sizeof(float), HT_MEM_RO);
    float *fC = hthread_malloc(0, M * N * sizeof(float), HT_MEM_WO);
    float *fC_cpu = calloc(M * N, sizeof(float));
    for (long i = 0; i < M * K; i++) fA[i] = (float)val(3 + i);
    for (long i = 0; i < K * N; i++) fB[i] = (float)val(5 + i);
    for (long i = 0; i < M * N; i++) fC[i] = 999.0f;
    unsigned long sargs[7] = {(unsigned long)M, (unsigned long)N, (unsigned long)K, (unsigned long)bid,
                              (unsigned long)fA, (unsigned long)fB, (unsigned long)fC};
    if (hthread_group_exec(tg, "launch_sgemm_NN", 4, 3, sargs) != 0) { printf("exec sgemm failed\n"); return 2; }
    hthread_group_wait(tg);
    const float alpha = 5.0f, beta = 3.0f;
    for (long i = 0; i < M; i++)
        for (long j = 0; j < N; j++) {
            for (long k = 0; k < K - K % K_G; k += K_G) {
                float tmp = 0.0f;
                for (long kk = 0; kk < K_G; kk++)
                    tmp = (float)fma((double)(alpha * fA[OFFSET(i, k + kk, K)]), (double)fB[OFFSET(k + kk, j, N)], (double)tmp);
                fC_cpu[OFFSET(i, j, N)] += tmp;
            }
            float tmp = 0.0f;
            for (long k = K - K % K_G; k < K; k++)
                tmp = (float)fma((double)(alpha * fA[OFFSET(i, k, K)]), (double)fB[OFFSET(k, j, N)], (double)tmp);
            fC_cpu[OFFSET(i, j, N)] += tmp;
            fC_cpu[OFFSET(i, j, N)] += beta;
        }
    long sbad = 0;
    for (long i = 0; i < M * N; i++) sbad += fC[i] != fC_cpu[i];
    printf("launch_sgemm_NN: %s (%ld mismatches)\n", sbad ? "Result Error!" : "Success!", sbad);
    fails += sbad != 0;

    /* transpose */
    unsigned long targs[5] = {(unsigned long)M, (unsigned long)K, (unsigned long)bid, (unsigned long)fA,
                              (unsigned long)fC_cpu};
    float *fT = hthread_malloc(0, M * K * sizeof(float), HT_MEM_WO);
    targs[4] = (unsigned long)fT;
    if (hthread_group_exec(tg, "transpose_float_32x32_dbuf", 3, 2, targs) != 0) { printf("exec transpose failed\n"); return 2; }
    hthread_group_wait(tg);
    long tbad = 0;
    for (long i = 0; i < M; i++)
        for (long j = 0; j < K; j++) tbad += fT[j * M + i] != fA[i * K + j];
    printf("transpose_float_32x32_dbuf: %s (%ld mismatches)\n", tbad ? "Result Error!" : "Success!", tbad);
    fails += tbad != 0;

    hthread_group_destroy(tg);
    hthread_barrier_destroy(bid);
    hthread_barrier_destroy(bid_T);
    hthread_dev_close(0);
    hthread_free(A); hthread_free(A_T); hthread_free(B); hthread_free(B_T);
    for (int m = 0; m < 4; m++) hthread_free(C[m]);
    hthread_free(fA); hthread_free(fB); hthread_free(fC); hthread_free(fT);
    free(C_cpu); free(fC_cpu);
    return fails ? 1 : 0;
}
