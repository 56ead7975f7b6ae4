/*
 * hthread_fake.c -- fake MT-3000 host runtime for compiling the reference's
 * host demos on this machine.  TEST INFRASTRUCTURE (fixture generation).
 *
 * hthread_group_exec(name, ...) runs the oracle restatement of the named
 * device kernel on the demo's buffers, with the argument packing of the
 * reference launchers:
 *   dgemm_release_V1.1/device_code/dgemm_launcher.c (lda,ldb,ldc,M,N,K,bid..,A,B,C)
 *   sgemm_release_V1.3.x/device_code/sgemm_launcher.c:11-37 (M,N,K,bid..,A,B,C;
 *       alpha=5, beta=3 as launcher globals)
 *   irr_*_launcher.c (M,N,K,bid..,A,B,C), irr_thinB_sgemm V1.2 alpha=5, beta=3
 *   transpose/host_code/transpose.c:73-77 (M,N,b_id,A,B)
 *   stencil_2d_V1.2/host_code/matrix_stencil.c:85-89 (M,N,A,B)
 * Compile-time switches: -DGBREF_SGEMM_ACCUM (sgemm V1.3.1 accumulates),
 * -DGBREF_THINB_V12 (irr_thinB_sgemm V1.2 alpha/beta + 3-level sum).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../oracle.h"

int   gbref_rand(void);
void *gbref_host_malloc(size_t n);

#define MAXBUF 64
static struct { void *p; size_t n; int host; } g_buf[MAXBUF];
static int g_nbuf = 0;
static uint64_t g_rand_ctr = 0;
static const uint64_t g_rand_seed = 0xC0FFEEULL;

static void track(void *p, size_t n, int host)
{
    if (g_nbuf < MAXBUF) { g_buf[g_nbuf].p = p; g_buf[g_nbuf].n = n; g_buf[g_nbuf].host = host; g_nbuf++; }
}

void *gbref_host_malloc(size_t n) { void *p = calloc(1, n); track(p, n, 1); return p; }

/* glibc RAND_MAX = 2^31-1; 31 bits of the SplitMix stream */
int gbref_rand(void)
{
    uint64_t z = gbo_mix64(gbo_mix64(g_rand_seed) + (g_rand_ctr + 1) * 0x9E3779B97F4A7C15ULL);
    g_rand_ctr++;
    return (int)(z >> 33);
}

void gbref_srand(unsigned seed) { (void)seed; g_rand_ctr = 0; }

int   hthread_dev_open(int dev_id) { (void)dev_id; return 0; }
int   hthread_dat_load(int dev_id, const char *name) { (void)dev_id; (void)name; return 0; }
void *hthread_malloc(int dev_id, size_t size, int flag) { (void)dev_id; (void)flag; void *p = calloc(1, size); track(p, size, 0); return p; }
void  hthread_free(void *ptr) { (void)ptr; }   /* dumped at dev_close; leak at exit */
int   hthread_barrier_create(int dev_id) { (void)dev_id; static int b = 0; return b++; }
void  hthread_barrier_destroy(int bid) { (void)bid; }
int   hthread_group_create(int dev_id, int nthreads) { (void)dev_id; (void)nthreads; return 1; }
int   hthread_group_wait(int tg_id) { (void)tg_id; return 0; }
void  hthread_group_destroy(int tg_id) { (void)tg_id; }

static int mode_of(const char *name, int *ta, int *tb)
{
    size_t L = strlen(name);
    if (L < 2) return -1;
    const char *m = name + L - 2;
    if (!strcmp(m, "NN")) { *ta = 0; *tb = 0; return 0; }
    if (!strcmp(m, "NT")) { *ta = 0; *tb = 1; return 0; }
    if (!strcmp(m, "TN")) { *ta = 1; *tb = 0; return 0; }
    if (!strcmp(m, "TT")) { *ta = 1; *tb = 1; return 0; }
    return -1;
}

int hthread_group_exec(int tg_id, const char *name, int n_scalar, int n_ptr, unsigned long *a)
{
    (void)tg_id; (void)n_ptr;
    int ta = 0, tb = 0;
    if (strstr(name, "null")) return 0;
    if (!strncmp(name, "launch_dgemm_", 13)) {                 /* dgemm V1.1 */
        if (mode_of(name, &ta, &tb)) return -1;
        long lda = a[0], ldb = a[1], ldc = a[2], M = a[3], N = a[4], K = a[5];
        double *A = (double *)a[n_scalar], *B = (double *)a[n_scalar + 1], *C = (double *)a[n_scalar + 2];
        gbo_dgemm_ref(ta, tb, M, N, K, A, lda, B, ldb, C, ldc, 512);
        return 0;
    }
    if (!strncmp(name, "launch_sgemm_", 13)) {                 /* sgemm V1.3.x */
        if (mode_of(name, &ta, &tb)) return -1;
        long M = a[0], N = a[1], K = a[2];
        float *A = (float *)a[n_scalar], *B = (float *)a[n_scalar + 1], *C = (float *)a[n_scalar + 2];
#ifdef GBREF_SGEMM_ACCUM
        int acc = 1;
#else
        int acc = 0;
#endif
        gbo_sgemm_ref(ta, tb, M, N, K, 5.0f, A, ta ? M : K, B, tb ? K : N, 3.0f, C, N, 512, acc);
        return 0;
    }
    if (!strncmp(name, "launch_irr_", 11)) {
        if (mode_of(name, &ta, &tb)) return -1;
        long M = a[0], N = a[1], K = a[2];
        long lda = ta ? M : K, ldb = tb ? K : N;
        if (strstr(name, "dgemm")) {
            gbo_dgemm_ref(ta, tb, M, N, K, (double *)a[n_scalar], lda, (double *)a[n_scalar + 1], ldb,
                          (double *)a[n_scalar + 2], N, 512);
        } else {
#ifdef GBREF_THINB_V12
            gbo_thinB_sgemm_ref(ta, tb, M, N, K, 5.0f, (float *)a[n_scalar], lda, (float *)a[n_scalar + 1], ldb,
                                3.0f, (float *)a[n_scalar + 2], N, 3072, 512, 0);
#else
            gbo_sgemm_irr_ref(ta, tb, M, N, K, (float *)a[n_scalar], lda, (float *)a[n_scalar + 1], ldb,
                              (float *)a[n_scalar + 2], N, 512);
#endif
        }
        return 0;
    }
    if (!strcmp(name, "transpose_float_32x32_dbuf")) {
        long M = a[0], N = a[1];
        gbo_transpose_f32(M, N, (float *)a[3], N, (float *)a[4], M);
        return 0;
    }
    if (!strcmp(name, "transpose_16x16_dbuf")) {
        long M = a[0], N = a[1];
        gbo_transpose_f64(M, N, (double *)a[3], N, (double *)a[4], M);
        return 0;
    }
    if (!strcmp(name, "stencil_vector") || !strcmp(name, "stencil_scalar")) {
        long M = a[0], N = a[1];
        /* one sweep A -> B (the demo's pointer swap is a no-op) */
        gbo_stencil_f64(M, N, (double *)a[2], (double *)a[3], 1, 0);
        return 0;
    }
    fprintf(stderr, "hthread_fake: unknown kernel %s\n", name);
    return -1;
}

/* Dump format: "GBREFDMP" u32 count, then per buffer: u32 host, u64 nbytes, bytes */
void hthread_dev_close(int dev_id)
{
    (void)dev_id;
    const char *path = getenv("GBREF_DUMP");
    if (!path) return;
    FILE *f = fopen(path, "wb");
    if (!f) return;
    fwrite("GBREFDMP", 1, 8, f);
    uint32_t cnt = (uint32_t)g_nbuf;
    fwrite(&cnt, 4, 1, f);
    for (int i = 0; i < g_nbuf; i++) {
        uint32_t h = (uint32_t)g_buf[i].host;
        uint64_t n = g_buf[i].n;
        fwrite(&h, 4, 1, f);
        fwrite(&n, 8, 1, f);
        fwrite(g_buf[i].p, 1, n, f);
    }
    fclose(f);
}
