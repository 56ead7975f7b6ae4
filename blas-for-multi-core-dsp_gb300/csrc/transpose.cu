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

// FP32: each thread moves 2 x 2 blocks, so the global reads (two rows of A)
// and writes (two rows of B) are 8-byte accesses like the FP64 kernel's.
// Needs lda, ldb even and 8-byte aligned bases; edges fall back to scalars.
constexpr int T2 = 64;
__global__ void __launch_bounds__(256) transpose2x2_kernel(const float *__restrict__ A, int64_t lda,
                                                           float *__restrict__ B, int64_t ldb, int64_t M, int64_t N) {
    __shared__ float tile[T2][T2 + 1];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;   // 32 x 8
    const int64_t r0 = (int64_t)blockIdx.y * T2, c0 = (int64_t)blockIdx.x * T2;
    const bool full = r0 + T2 <= M && c0 + T2 <= N;
#pragma unroll
    for (int i = 0; i < T2; i += 16) {
        const int rr = ty * 2 + i, cc = tx * 2;
        const int64_t r = r0 + rr, c = c0 + cc;
        if (full) {
            float2 u = *reinterpret_cast<const float2 *>(A + r * lda + c);
            float2 v = *reinterpret_cast<const float2 *>(A + (r + 1) * lda + c);
            tile[rr][cc] = u.x; tile[rr][cc + 1] = u.y;
            tile[rr + 1][cc] = v.x; tile[rr + 1][cc + 1] = v.y;
        } else {
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int b = 0; b < 2; b++)
                    if (r + a < M && c + b < N) tile[rr + a][cc + b] = A[(r + a) * lda + c + b];
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < T2; i += 16) {
        const int bc = ty * 2 + i, br = tx * 2;   // B row c0+bc (+1), columns r0+br (+1)
        const int64_t row = c0 + bc, col = r0 + br;
        if (full) {
            *reinterpret_cast<float2 *>(B + row * ldb + col) = make_float2(tile[br][bc], tile[br + 1][bc]);
            *reinterpret_cast<float2 *>(B + (row + 1) * ldb + col) = make_float2(tile[br][bc + 1], tile[br + 1][bc + 1]);
        } else {
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int b = 0; b < 2; b++)
                    if (row + a < N && col + b < M) B[(row + a) * ldb + col + b] = tile[br + b][bc + a];
        }
    }
}

// B += A^T (transpose-accumulate): the 64 x 64 tile of A goes through padded
// shared memory as above; each B element gets one IEEE add.  HBM-bound:
// 3 M N sizeof(T) bytes (A read, B read and written).
template <typename T>
__global__ void __launch_bounds__(TILE * ROWS) transpose_add_kernel(const T *__restrict__ A, int64_t lda, T *B,
                                                                    int64_t ldb, int64_t M, int64_t N) {
    __shared__ T tile[TILE][TILE + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t r0 = (int64_t)blockIdx.y * TILE, c0 = (int64_t)blockIdx.x * TILE;
#pragma unroll
    for (int i = 0; i < TILE; i += ROWS) {
        int64_t r = r0 + ty + i, c = c0 + tx;
        if (r < M && c < N) tile[ty + i][tx] = A[r * lda + c];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < TILE; i += ROWS) {
        int64_t br = c0 + ty + i, bc = r0 + tx;
        if (br < N && bc < M) B[br * ldb + bc] = B[br * ldb + bc] + tile[tx][ty + i];
    }
}

template <typename T>
gb_status transpose_add(int64_t M, int64_t N, const T *A, int64_t lda, T *B, int64_t ldb, void *stream) {
    GB_CHECK_ARG(M >= 0 && N >= 0, "transpose_add: negative size");
    GB_CHECK_ARG(lda >= N || M == 0, "transpose_add: lda (%lld) < N (%lld)", (long long)lda, (long long)N);
    GB_CHECK_ARG(ldb >= M || N == 0, "transpose_add: ldb (%lld) < M (%lld)", (long long)ldb, (long long)M);
    if (M == 0 || N == 0) return ok();
    GB_CHECK_ARG(A && B, "transpose_add: null pointer");
    GB_CHECK_ARG((const void *)A != (const void *)B, "transpose_add: A and B must not be the same buffer");
    dim3 grid((unsigned)ceil_div(N, TILE), (unsigned)ceil_div(M, TILE));
    GB_CHECK_ARG(grid.y <= 65535u, "transpose_add: M too large");
    transpose_add_kernel<T><<<grid, dim3(TILE, ROWS), 0, as_stream(stream)>>>(A, lda, B, ldb, M, N);
    GB_LAUNCH_CHECK("transpose_add_kernel");
    return ok();
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
    if (sizeof(T) == 4 && lda % 2 == 0 && ldb % 2 == 0 && (uintptr_t)A % 8 == 0 && (uintptr_t)B % 8 == 0) {
        transpose2x2_kernel<<<grid, 256, 0, as_stream(stream)>>>((const float *)A, lda, (float *)B, ldb, M, N);
        GB_LAUNCH_CHECK("transpose2x2_kernel");
        return ok();
    }
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

gb_status gb_transpose_add_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb,
                               void *stream) {
    return gb::transpose_add<float>(M, N, A, lda, B, ldb, stream);
}

gb_status gb_transpose_add_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb,
                               void *stream) {
    return gb::transpose_add<double>(M, N, A, lda, B, ldb, stream);
}

}  // extern "C"
