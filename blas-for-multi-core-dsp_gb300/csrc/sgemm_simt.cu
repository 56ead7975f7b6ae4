// sgemm_simt.cu -- plain FP32 SGEMM on the CUDA cores (FFMA register tiles).
//
// The GB300 counterpart of the reference's r6c96/r6c128 FP32 micro-kernels
// (sgemm_release_V1.3.2/device_code/sgemm_kernel.c:984-2474) and their
// blocked drivers (sgemm_NN_qxx :2476, sgemm_NT_qxx :2998, sgemm_TN_qxx
// :4029, sgemm_TT_qxx :4043).  op(A)/op(B) are absorbed into the tile
// loaders (no transpose pass): each mode reads its operand along the
// contiguous dimension with 128-bit loads and writes the K-major shared
// tile the FFMA loop wants.
//
// 128x128 C tile per CTA, K step 8, 256 threads with an 8x8 register tile
// each, shared memory double-buffered with the next tile prefetched into
// registers while the current one is consumed.  alpha/beta are applied in
// the epilogue (BLAS, scalar-beta or accumulate semantics).
#include "gb_common.cuh"
#include "sm100_ptx.cuh"

namespace gb {
namespace {

constexpr int BM = 128, BN = 128, BK = 8, NT = 256;

struct SimtParams {
    int64_t M, N, K, lda, ldb, ldc;
    float alpha, beta;
    int semantics;
};

// Load the k-tile [k0, k0+8) of op(A) (128 x 8) into registers.
template <bool TA, bool VEC>
__device__ __forceinline__ void ldg_a(const float *__restrict__ A, const SimtParams &p, int64_t m0, int64_t k0,
                                      float (&r)[4]) {
    const int tid = threadIdx.x;
    if (!TA) {  // A is M x K, k contiguous: row = tid/2, 4 k's
        int64_t m = m0 + tid / 2, k = k0 + (tid % 2) * 4;
        if (VEC && m < p.M && k + 3 < p.K) {
            float4 v = *reinterpret_cast<const float4 *>(A + m * p.lda + k);
            r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = (m < p.M && k + i < p.K) ? A[m * p.lda + k + i] : 0.f;
        }
    } else {    // A is K x M, m contiguous: k = tid/32, 4 m's
        int64_t k = k0 + tid / 32, m = m0 + (tid % 32) * 4;
        if (VEC && k < p.K && m + 3 < p.M) {
            float4 v = *reinterpret_cast<const float4 *>(A + k * p.lda + m);
            r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = (k < p.K && m + i < p.M) ? A[k * p.lda + m + i] : 0.f;
        }
    }
}

template <bool TA>
__device__ __forceinline__ void sts_a(float (*As)[BM + 4], const float (&r)[4]) {
    const int tid = threadIdx.x;
    if (!TA) {
        int mm = tid / 2, kk = (tid % 2) * 4;
#pragma unroll
        for (int i = 0; i < 4; i++) As[kk + i][mm] = r[i];
    } else {
        int kk = tid / 32, mm = (tid % 32) * 4;
        *reinterpret_cast<float4 *>(&As[kk][mm]) = make_float4(r[0], r[1], r[2], r[3]);
    }
}

// op(B) k-tile (8 x 128).
template <bool TB, bool VEC>
__device__ __forceinline__ void ldg_b(const float *__restrict__ B, const SimtParams &p, int64_t n0, int64_t k0,
                                      float (&r)[4]) {
    const int tid = threadIdx.x;
    if (!TB) {  // B is K x N, n contiguous
        int64_t k = k0 + tid / 32, n = n0 + (tid % 32) * 4;
        if (VEC && k < p.K && n + 3 < p.N) {
            float4 v = *reinterpret_cast<const float4 *>(B + k * p.ldb + n);
            r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = (k < p.K && n + i < p.N) ? B[k * p.ldb + n + i] : 0.f;
        }
    } else {    // B is N x K, k contiguous
        int64_t n = n0 + tid / 2, k = k0 + (tid % 2) * 4;
        if (VEC && n < p.N && k + 3 < p.K) {
            float4 v = *reinterpret_cast<const float4 *>(B + n * p.ldb + k);
            r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) r[i] = (n < p.N && k + i < p.K) ? B[n * p.ldb + k + i] : 0.f;
        }
    }
}

template <bool TB>
__device__ __forceinline__ void sts_b(float (*Bs)[BN + 4], const float (&r)[4]) {
    const int tid = threadIdx.x;
    if (!TB) {
        int kk = tid / 32, nn = (tid % 32) * 4;
        *reinterpret_cast<float4 *>(&Bs[kk][nn]) = make_float4(r[0], r[1], r[2], r[3]);
    } else {
        int nn = tid / 2, kk = (tid % 2) * 4;
#pragma unroll
        for (int i = 0; i < 4; i++) Bs[kk + i][nn] = r[i];
    }
}

template <bool TA, bool TB, bool VEC>
__global__ void __launch_bounds__(NT, 2) sgemm_simt_kernel(const float *__restrict__ A, const float *__restrict__ B,
                                                           float *__restrict__ C, SimtParams p) {
    __shared__ __align__(16) float As[2][BK][BM + 4];
    __shared__ __align__(16) float Bs[2][BK][BN + 4];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;

    // acc[i][jj]: the outputs (i, 2jj) and (i, 2jj + 1) as one packed FP32x2 register; each output
    // still sees its own FMAs in k order, so results equal one FFMA per product
    uint64_t acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int jj = 0; jj < 4; jj++) acc[i][jj] = 0ull;

    float ra[4], rb[4];
    ldg_a<TA, VEC>(A, p, m0, 0, ra);
    ldg_b<TB, VEC>(B, p, n0, 0, rb);
    sts_a<TA>(As[0], ra);
    sts_b<TB>(Bs[0], rb);
    __syncthreads();

    const int64_t ktiles = ceil_div(p.K, BK);
    for (int64_t kt = 0; kt < ktiles; kt++) {
        const int cur = kt & 1;
        const bool more = kt + 1 < ktiles;
        if (more) {
            ldg_a<TA, VEC>(A, p, m0, (kt + 1) * BK, ra);
            ldg_b<TB, VEC>(B, p, n0, (kt + 1) * BK, rb);
        }
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            float a[8];
            float4 a0 = *reinterpret_cast<const float4 *>(&As[cur][kk][ty * 4]);
            float4 a1 = *reinterpret_cast<const float4 *>(&As[cur][kk][64 + ty * 4]);
            float4 b0 = *reinterpret_cast<const float4 *>(&Bs[cur][kk][tx * 4]);
            float4 b1 = *reinterpret_cast<const float4 *>(&Bs[cur][kk][64 + tx * 4]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
            a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
            const uint64_t b2[4] = {ptx::f2_pack(b0.x, b0.y), ptx::f2_pack(b0.z, b0.w), ptx::f2_pack(b1.x, b1.y),
                                    ptx::f2_pack(b1.z, b1.w)};
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const uint64_t ai = ptx::f2_pack(a[i], a[i]);
#pragma unroll
                for (int jj = 0; jj < 4; jj++) acc[i][jj] = ptx::f2_fma_rn(ai, b2[jj], acc[i][jj]);
            }
        }
        if (more) {
            sts_a<TA>(As[cur ^ 1], ra);
            sts_b<TB>(Bs[cur ^ 1], rb);
        }
        __syncthreads();
    }

    // epilogue
#pragma unroll
    for (int i = 0; i < 8; i++) {
        int64_t m = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (m >= p.M) continue;
        float accf[8];
#pragma unroll
        for (int jj = 0; jj < 4; jj++) ptx::f2_unpack(acc[i][jj], accf[2 * jj], accf[2 * jj + 1]);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            int64_t n = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            if (n >= p.N) continue;
            float *cp = C + m * p.ldc + n;
            float v = p.alpha * accf[j];
            if (p.semantics == GB_SEM_BLAS) {
                if (p.beta != 0.f) v = fmaf(p.beta, *cp, v);
            } else if (p.semantics == GB_SEM_SCALAR_BETA) {
                v = v + p.beta;
            } else {
                v = *cp + (v + p.beta);
            }
            *cp = v;
        }
    }
}

template <bool TA, bool TB>
gb_status launch_mode(const GemmArgs &g, const SimtParams &p, bool vec) {
    dim3 grid((unsigned)ceil_div(g.N, BN), (unsigned)ceil_div(g.M, BM));
    if (vec)
        sgemm_simt_kernel<TA, TB, true><<<grid, NT, 0, g.stream>>>((const float *)g.A, (const float *)g.B,
                                                                   (float *)g.C, p);
    else
        sgemm_simt_kernel<TA, TB, false><<<grid, NT, 0, g.stream>>>((const float *)g.A, (const float *)g.B,
                                                                    (float *)g.C, p);
    GB_LAUNCH_CHECK("sgemm_simt_kernel");
    return ok();
}

}  // namespace

gb_status launch_sgemm_simt(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    if (ceil_div(g.M, BM) > 65535) return set_status(GB_ERR_UNSUPPORTED, "simt sgemm: M too large");
    SimtParams p{g.M, g.N, g.K, g.lda, g.ldb, g.ldc, (float)g.alpha, (float)g.beta, g.semantics};
    bool vec = (g.lda % 4 == 0) && (g.ldb % 4 == 0) && ((uintptr_t)g.A % 16 == 0) && ((uintptr_t)g.B % 16 == 0);
    if (!g.ta && !g.tb) return launch_mode<false, false>(g, p, vec);
    if (!g.ta && g.tb) return launch_mode<false, true>(g, p, vec);
    if (g.ta && !g.tb) return launch_mode<true, false>(g, p, vec);
    return launch_mode<true, true>(g, p, vec);
}

}  // namespace gb
