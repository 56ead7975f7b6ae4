/* Compiles and links (never runs) one call of each family of the C ABI, as a
 * reference-side host program would write them: the headers must stay valid
 * C99 and C++ with every warning an error. */
#include <stddef.h>
#include <stdint.h>

#include "gbblas.h"
#include "gbblas_ref.h"

int gbblas_abi_compile_check(float *fA, float *fB, float *fC, double *dA, double *dB, double *dC, void *stream) {
    gb_gemm_opts o;
    gb_gemm_opts_init(&o);
    o.algo = GB_ALGO_BF16X3;
    o.stream = stream;
    int bad = 0;
    bad |= gb_sgemm('N', 'T', 64, 64, 64, 1.5f, fA, 64, fB, 64, -0.5f, fC, 64, &o) != GB_OK;
    o.algo = GB_ALGO_OZAKI;
    o.ozaki_slices = 0;
    o.target_err = 0.0;
    bad |= gb_dgemm('T', 'N', 64, 64, 64, 1.0, dA, 64, dB, 64, 1.0, dC, 64, &o) != GB_OK;
    bad |= gb_sgemm_skinny_noalloc('N', 'N', 4096, 8, 64, 1.0f, fA, 64, fB, 8, 0.0f, fC, 8, GB_SEM_BLAS, stream) != GB_OK;
    bad |= gb_gemm_pick_algo(64, 'N', 'N', 8192, 8192, 8192) < 0;
    bad |= gb_gemm_strided_batched(32, 'N', 'N', 16, 16, 16, 1.0, fA, 16, 256, fB, 16, 256, 0.0, fC, 16, 256, 4,
                                   GB_SEM_BLAS, stream) != GB_OK;
    bad |= gb_transpose_f32(64, 32, fA, 32, fB, 64, stream) != GB_OK;
    bad |= gb_transpose_add_f64(64, 32, dA, 32, dB, 64, stream) != GB_OK;
    bad |= gb_stencil2d_f64(62, 62, dA, dB, 10, 0, stream) != GB_OK;
    const float w[9] = {0, 0.25f, 0, 0.25f, 0, 0.25f, 0, 0.25f, 0};
    bad |= gb_stencil9_f32(62, 62, fA, fB, 10, w, stream) != GB_OK;
    bad |= gb_sync(stream) != GB_OK;
    unsigned long args[7] = {64, 64, 64, 0, (unsigned long)(uintptr_t)fA, (unsigned long)(uintptr_t)fB,
                             (unsigned long)(uintptr_t)fC};
    bad |= gb_exec("launch_sgemm_NN", 4, 3, args) != GB_OK;
    dgemm_NN(64, 64, 64, 64, 64, 64, 0, dA, dB, dC);
    gb_ref_set_algo(GB_ALGO_ORDERED);
    return bad || gb_last_error() == NULL;
}

int main(int argc, char **argv) {
    (void)argv;
    /* never runs the calls: the check is that this compiles and links */
    if (argc > 100) return gbblas_abi_compile_check(NULL, NULL, NULL, NULL, NULL, NULL, NULL);
    return 0;
}
