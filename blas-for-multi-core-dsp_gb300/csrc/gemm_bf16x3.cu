// gemm_bf16x3.cu -- SGEMM as three BF16 products on the tcgen05 tensor cores.
//
// C = alpha * op(A) op(B) (+ beta C / + beta), FP32 in and out.  Each FP32
// operand x is split into x_hi = bf16(x) and x_lo = bf16(x - x_hi); the
// product is accumulated in FP32 in tensor memory as
//     a_hi*b_hi + a_hi*b_lo + a_lo*b_hi
// (the a_lo*b_lo term, ~2^-16 relative, is dropped).  This is the precision
// form of the reference's FP32 SGEMM (sgemm_release_V1.3.2/device_code/
// sgemm_kernel.c:2476-4505); it has no counterpart in the reference.
//
// Two kernels:
//  1. split: op(A) -> A_hi, A_lo (M x Kp, K-major BF16), op(B) -> B_hi, B_lo
//     (N x Kp, K-major), Kp = K rounded up to 64 with zeros.  The transpose
//     modes are absorbed here (a row-major or a transposed read, always a
//     K-major write), so the GEMM kernel has one operand layout.
//  2. gemm: one 128 x 256 C tile per CTA, K in blocks of 64 (one 128-byte
//     swizzle atom), a 2-stage TMA -> shared memory pipeline with mbarriers;
//     warp 0 issues TMA, warp 1 issues tcgen05.mma (M=128, N=256, K=16, three
//     products per K step into one TMEM accumulator of 256 columns), warps
//     2-5 read the accumulator with tcgen05.ld and apply alpha/beta.
#include <cuda.h>
#include <cuda_bf16.h>

#include "gb_common.cuh"
#include "sm100_ptx.cuh"

namespace gb {

// TMA descriptor encoding through the driver entry point (no -lcuda).
typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                    CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                    CUtensorMapFloatOOBfill);

static PFN_encodeTiled encode_fn() {
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_encodeTiled)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// 2-D BF16 tensor [outer][inner] (inner contiguous), box box_inner x box_outer,
// 128-byte swizzle.  Returns false if the encoder rejects it.
bool make_tmap_bf16_sw128(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer,
                          uint64_t row_bytes, uint32_t box_inner, uint32_t box_outer) {
    PFN_encodeTiled enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

namespace {

// ------------------------------------------------------------------ split
// out_hi/out_lo: rows x kp (K-major).  Source element (r, k):
// trans ? X[k*ldx + r] : X[r*ldx + k].  32x32 tiles through shared memory
// so both the read and the write are coalesced in either layout.
__global__ void __launch_bounds__(256) split_kernel(const float *__restrict__ X, int64_t ldx, int trans, int64_t rows,
                                                    int64_t K, int64_t kp, __nv_bfloat16 *__restrict__ out_hi,
                                                    __nv_bfloat16 *__restrict__ out_lo) {
    __shared__ float tile[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;   // 32 x 8
    const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
#pragma unroll
    for (int i = 0; i < 32; i += 8) {
        float v = 0.f;
        if (trans) {   // coalesced along r: tile[k][r]
            int64_t k = k0 + ty + i, r = r0 + tx;
            if (k < K && r < rows) v = X[k * ldx + r];
            tile[ty + i][tx] = v;
        } else {       // coalesced along k: tile[k][r] via transposed store
            int64_t r = r0 + ty + i, k = k0 + tx;
            if (k < K && r < rows) v = X[r * ldx + k];
            tile[tx][ty + i] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 32; i += 8) {
        int64_t r = r0 + ty + i, k = k0 + tx;
        if (r < rows && k < kp) {
            float x = tile[tx][ty + i];
            __nv_bfloat16 h = __float2bfloat16_rn(x);
            __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
            out_hi[r * kp + k] = h;
            out_lo[r * kp + k] = l;
        }
    }
}

// ------------------------------------------------------------------- gemm
constexpr int BM = 128, BN = 256, BK = 64, STAGES = 2;
constexpr int A_TILE = BM * BK * 2;            // 16 KB
constexpr int B_TILE = BN * BK * 2;            // 32 KB
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int NT = 192;
constexpr uint32_t TMEM_COLS = 256;

struct EpiParams {
    float *C;
    int64_t M, N, ldc;
    float alpha, beta;
    int semantics;
    int num_kb;
    int *err;
};

__global__ void __launch_bounds__(NT, 1)
    bf16x3_gemm_kernel(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                       const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
                       EpiParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *accb = empty + STAGES;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accb + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1);
        }
        ptx::mbar_init(accb, 1);
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&tmAh);
        ptx::tma_prefetch_desc(&tmAl);
        ptx::tma_prefetch_desc(&tmBh);
        ptx::tma_prefetch_desc(&tmBl);
    }
    if (warp == 1) ptx::tmem_alloc(tmem_slot, TMEM_COLS);
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {   // TMA producer
            for (int kb = 0; kb < p.num_kb; kb++) {
                const int s = kb % STAGES;
                if (kb >= STAGES && !ptx::mbar_wait(&empty[s], ((kb / STAGES) & 1) ^ 1, p.err, 1)) break;
                uint8_t *st = smem + s * STAGE_BYTES;
                ptx::mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
                ptx::tma_load_2d(st, &tmAh, &full[s], kb * BK, m0);
                ptx::tma_load_2d(st + A_TILE, &tmAl, &full[s], kb * BK, m0);
                ptx::tma_load_2d(st + 2 * A_TILE, &tmBh, &full[s], kb * BK, n0);
                ptx::tma_load_2d(st + 2 * A_TILE + B_TILE, &tmBl, &full[s], kb * BK, n0);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, BN);
            bool okk = true;
            for (int kb = 0; kb < p.num_kb; kb++) {
                const int s = kb % STAGES;
                if (!ptx::mbar_wait(&full[s], (kb / STAGES) & 1, p.err, 2)) { okk = false; break; }
                ptx::tc_fence_after();
                const uint32_t st = ptx::smem_u32(smem + s * STAGE_BYTES);
                const uint64_t ah = ptx::sdesc_kmajor_sw128(st);
                const uint64_t al = ptx::sdesc_kmajor_sw128(st + A_TILE);
                const uint64_t bh = ptx::sdesc_kmajor_sw128(st + 2 * A_TILE);
                const uint64_t bl = ptx::sdesc_kmajor_sw128(st + 2 * A_TILE + B_TILE);
#pragma unroll
                for (int k = 0; k < BK / 16; k++) {
                    // advance 16 BF16 = 32 bytes along K inside the swizzle atom
                    const uint64_t dk = (uint64_t)((k * 32) >> 4);
                    ptx::umma_f16(tmem, al + dk, bh + dk, idesc, (kb | k) != 0);
                    ptx::umma_f16(tmem, ah + dk, bl + dk, idesc, 1);
                    ptx::umma_f16(tmem, ah + dk, bh + dk, idesc, 1);
                }
                ptx::umma_commit(&empty[s]);
            }
            if (okk) ptx::umma_commit(accb);
        }
    } else {               // epilogue: warps 2..5 own TMEM lane quarters (warp % 4)
        const int q = warp % 4;
        const bool okw = ptx::mbar_wait(accb, 0, p.err, 3);
        ptx::tc_fence_after();
        if (okw) {
            const int64_t row = (int64_t)m0 + q * 32 + lane;
            for (int c = 0; c < BN; c += 32) {
                uint32_t r[32];
                ptx::tmem_ld_32x32b_x32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, r);
                ptx::tmem_ld_wait();
                if (row < p.M) {
                    float *crow = p.C + row * p.ldc + n0 + c;
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        if (n0 + c + j < p.N) {
                            float v = p.alpha * __uint_as_float(r[j]);
                            if (p.semantics == GB_SEM_BLAS) {
                                if (p.beta != 0.f) v = fmaf(p.beta, crow[j], v);
                            } else if (p.semantics == GB_SEM_SCALAR_BETA) {
                                v = v + p.beta;
                            } else {
                                v = crow[j] + (v + p.beta);
                            }
                            crow[j] = v;
                        }
                    }
                }
            }
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

}  // namespace

gb_status launch_sgemm_bf16x3(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    if (g.M > 0x7fffffff / 2 || g.N > 0x7fffffff / 2 || g.K > 0x7fffffff / 2)
        return set_status(GB_ERR_UNSUPPORTED, "bf16x3: dimension too large");
    const int64_t kp = ceil_div(g.K, BK) * BK;
    const size_t a_bytes = (size_t)g.M * kp * 2, b_bytes = (size_t)g.N * kp * 2;
    uint8_t *ws = (uint8_t *)workspace(2 * a_bytes + 2 * b_bytes + 4096, g.stream);
    if (!ws) return (gb_status)gb_get_last_status();
    __nv_bfloat16 *ah = (__nv_bfloat16 *)ws;
    __nv_bfloat16 *al = (__nv_bfloat16 *)(ws + a_bytes);
    __nv_bfloat16 *bh = (__nv_bfloat16 *)(ws + 2 * a_bytes);
    __nv_bfloat16 *bl = (__nv_bfloat16 *)(ws + 2 * a_bytes + b_bytes);
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "bf16x3: no device error word");

    // split: op(A)(m, k) = ta ? A[k*lda + m] : A[m*lda + k]
    //        op(B)^T(n, k) = op(B)(k, n) = tb ? B[n*ldb + k] : B[k*ldb + n]
    dim3 sgA((unsigned)ceil_div(kp, 32), (unsigned)ceil_div(g.M, 32));
    dim3 sgB((unsigned)ceil_div(kp, 32), (unsigned)ceil_div(g.N, 32));
    if (sgA.y > 65535u || sgB.y > 65535u) return set_status(GB_ERR_UNSUPPORTED, "bf16x3: M or N too large");
    split_kernel<<<sgA, 256, 0, g.stream>>>((const float *)g.A, g.lda, g.ta ? 1 : 0, g.M, g.K, kp, ah, al);
    GB_LAUNCH_CHECK("bf16x3 split A");
    split_kernel<<<sgB, 256, 0, g.stream>>>((const float *)g.B, g.ldb, g.tb ? 0 : 1, g.N, g.K, kp, bh, bl);
    GB_LAUNCH_CHECK("bf16x3 split B");

    CUtensorMap tAh, tAl, tBh, tBl;
    bool okm = make_tmap_bf16_sw128(&tAh, ah, kp, g.M, kp * 2, BK, BM) &&
               make_tmap_bf16_sw128(&tAl, al, kp, g.M, kp * 2, BK, BM) &&
               make_tmap_bf16_sw128(&tBh, bh, kp, g.N, kp * 2, BK, BN) &&
               make_tmap_bf16_sw128(&tBl, bl, kp, g.N, kp * 2, BK, BN);
    if (!okm) return set_status(GB_ERR_CUDA, "bf16x3: cuTensorMapEncodeTiled failed");

    static bool attr_set = false;
    if (!attr_set) {
        GB_CUDA_TRY(cudaFuncSetAttribute(bf16x3_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        attr_set = true;
    }
    EpiParams p{(float *)g.C, g.M, g.N, g.ldc, (float)g.alpha, (float)g.beta, g.semantics, (int)(kp / BK), err};
    dim3 grid((unsigned)ceil_div(g.N, BN), (unsigned)ceil_div(g.M, BM));
    bf16x3_gemm_kernel<<<grid, NT, SMEM_BYTES, g.stream>>>(tAh, tAl, tBh, tBl, p);
    GB_LAUNCH_CHECK("bf16x3_gemm_kernel");
    return ok();
}

}  // namespace gb
