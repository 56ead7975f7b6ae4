// dgemm_dmma.cu -- DGEMM on the FP64 tensor pipe (mma.sync m8n8k4 f64).
//
// The GB300 counterpart of the reference's FP64 micro-kernels
// micro_kernel_asm_r6c64 / r6c48 (dgemm_release_V1.1/device_code/
// dgemm_kernel.c:1478, :1090) and the drivers dgemm_NN/NT/TN/TT (:1994,
// :2247, :2896, :2912).  64x64 C tile per CTA, 4 warps of 32x32 (4x4 DMMA
// tiles each), K staged 16 at a time through shared memory; op(A)/op(B)
// are absorbed into the tile loaders.  The DMMA sums four products per
// step, so results differ from the reference order in the last bits (the
// ORDERED algorithm is the bit-exact one); accuracy is the usual
// normwise ~K*u64.
#include "gb_common.cuh"

namespace gb {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 128;

struct DmmaParams {
    int64_t M, N, K, lda, ldb, ldc;
    int ta, tb;
    double alpha, beta;
    int semantics;
};

__device__ __forceinline__ void dmma_8x8x4(double &d0, double &d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(NT) dgemm_dmma_kernel(const double *__restrict__ A, const double *__restrict__ B,
                                                        double *__restrict__ C, DmmaParams p) {
    __shared__ double As[BK][BM + 2];
    __shared__ double Bs[BK][BN + 2];
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const int wm = (warp / 2) * 32, wn = (warp % 2) * 32;
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;

    double acc[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j][0] = acc[i][j][1] = 0.0;

    for (int64_t k0 = 0; k0 < p.K; k0 += BK) {
        __syncthreads();
#pragma unroll
        for (int r = 0; r < (BM * BK) / NT; r++) {
            int l = tid + r * NT, mm, kk;
            if (p.ta) { mm = l % BM; kk = l / BM; } else { mm = l / BK; kk = l % BK; }
            int64_t m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < p.M && k < p.K) ? (p.ta ? A[k * p.lda + m] : A[m * p.lda + k]) : 0.0;
        }
#pragma unroll
        for (int r = 0; r < (BN * BK) / NT; r++) {
            int l = tid + r * NT, nn, kk;
            if (p.tb) { nn = l / BK; kk = l % BK; } else { nn = l % BN; kk = l / BN; }
            int64_t n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < p.N && k < p.K) ? (p.tb ? B[n * p.ldb + k] : B[k * p.ldb + n]) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 4) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[ks + lane % 4][wm + i * 8 + lane / 4];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[ks + lane % 4][wn + j * 8 + lane / 4];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) dmma_8x8x4(acc[i][j][0], acc[i][j][1], a[i], b[j]);
        }
    }

#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                int64_t m = m0 + wm + i * 8 + lane / 4;
                int64_t n = n0 + wn + j * 8 + 2 * (lane % 4) + h;
                if (m >= p.M || n >= p.N) continue;
                double *cp = C + m * p.ldc + n;
                double v = p.alpha * acc[i][j][h];
                if (p.semantics == GB_SEM_BLAS) {
                    if (p.beta != 0.0) v = fma(p.beta, *cp, v);
                } else if (p.semantics == GB_SEM_SCALAR_BETA) {
                    v = v + p.beta;
                } else {
                    v = *cp + (v + p.beta);
                }
                *cp = v;
            }
}

}  // namespace

gb_status launch_dgemm_dmma(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    dim3 grid((unsigned)ceil_div(g.N, BN), (unsigned)ceil_div(g.M, BM));
    if (grid.y > 65535u) return set_status(GB_ERR_UNSUPPORTED, "dmma dgemm: M too large");
    DmmaParams p{g.M, g.N, g.K, g.lda, g.ldb, g.ldc, g.ta, g.tb, g.alpha, g.beta, g.semantics};
    dgemm_dmma_kernel<<<grid, NT, 0, g.stream>>>((const double *)g.A, (const double *)g.B, (double *)g.C, p);
    GB_LAUNCH_CHECK("dgemm_dmma_kernel");
    return ok();
}

}  // namespace gb
