// transpose.cu -- out-of-place matrix transpose, bit-exact copy.
//
// Replaces transpose_float_32x32_dbuf / transpose_16x16_dbuf
// (transpose/device_code/kernel.c:2002, :1167) and the ld-aware
// transpose_A2B (dgemm_release_V1.1/device_code/dgemm_kernel.c:974): B (N x M,
// ldb) = A^T with A M x N (lda).  The reference moves 128x128 tiles through
// on-chip AM with double-buffered DMA and transposes 32x32 / 16x16 blocks in
// registers; here a CTA stages a 64x64 tile through padded shared memory so
// both the HBM read (rows of A) and the write (rows of B) are coalesced.
// HBM-bound: 2*M*N*sizeof(T) bytes.
#include "gb_common.cuh"

namespace gb {
namespace {

constexpr int TILE = 64, ROWS = 16;   // 64 x 16 threads, 4 rows each

template <typename T>
__global__ void __launch_bounds__(TILE * ROWS) transpose_kernel(const T *__restrict__ A, int64_t lda,
                                                                T *__restrict__ B, int64_t ldb, int64_t M,
                                                                int64_t N) {
    __shared__ T tile[TILE][TILE + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t r0 = (int64_t)blockIdx.y * TILE, c0 = (int64_t)blockIdx.x * TILE;
    // read a 64x64 tile of A: rows r0.., columns c0.. (coalesced along columns)
#pragma unroll
    for (int i = 0; i < TILE; i += ROWS) {
        int64_t r = r0 + ty + i, c = c0 + tx;
        if (r < M && c < N) tile[ty + i][tx] = A[r * lda + c];
    }
    __syncthreads();
    // write B rows c0.. (= A columns), columns r0.. (coalesced along B's rows)
#pragma unroll
    for (int i = 0; i < TILE; i += ROWS) {
        int64_t br = c0 + ty + i, bc = r0 + tx;
        if (br < N && bc < M) B[br * ldb + bc] = tile[tx][ty + i];
    }
}

template <typename T>
gb_status transpose(int64_t M, int64_t N, const T *A, int64_t lda, T *B, int64_t ldb, void *stream) {
    GB_CHECK_ARG(M >= 0 && N >= 0, "transpose: negative size");
    GB_CHECK_ARG(lda >= N || M == 0, "transpose: lda (%lld) < N (%lld)", (long long)lda, (long long)N);
    GB_CHECK_ARG(ldb >= M || N == 0, "transpose: ldb (%lld) < M (%lld)", (long long)ldb, (long long)M);
    if (M == 0 || N == 0) return ok();
    GB_CHECK_ARG(A && B, "transpose: null pointer");
    GB_CHECK_ARG((const void *)A != (const void *)B, "transpose: in-place transpose is not supported");
    dim3 grid((unsigned)ceil_div(N, TILE), (unsigned)ceil_div(M, TILE));
    GB_CHECK_ARG(grid.y <= 65535u, "transpose: M too large");
    transpose_kernel<T><<<grid, dim3(TILE, ROWS), 0, as_stream(stream)>>>(A, lda, B, ldb, M, N);
    GB_LAUNCH_CHECK("transpose_kernel");
    return ok();
}

}  // namespace
}  // namespace gb

extern "C" {

gb_status gb_transpose_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb, void *stream) {
    return gb::transpose<float>(M, N, A, lda, B, ldb, stream);
}

gb_status gb_transpose_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb,
                           void *stream) {
    return gb::transpose<double>(M, N, A, lda, B, ldb, stream);
}

}  // extern "C"
