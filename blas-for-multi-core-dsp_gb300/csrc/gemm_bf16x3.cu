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
//  2. gemm: persistent, one CTA per SM over 128 x 256 C tiles, K in blocks of
//     32 (one 64-byte swizzle atom), a 4-stage TMA -> shared memory pipeline
//     with mbarriers; warp 0 issues TMA, warp 1 issues tcgen05.mma (M=128,
//     N=256, K=16, three products per K step into a TMEM accumulator of 256
//     columns, two accumulators alternating between tiles), warps 2-5 read
//     the finished accumulator with tcgen05.ld, stage it through shared memory
//     and write C row-contiguously with alpha/beta applied.
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
// 64- or 128-byte swizzle.  Returns false if the encoder rejects it.
bool make_tmap_bf16(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                    uint32_t box_inner, uint32_t box_outer, int swizzle_bytes) {
    PFN_encodeTiled enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE,
                     swizzle_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
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
// Persistent: one CTA per SM walks the 128 x 256 C tiles in a grouped order
// (GROUP_M tile rows at a time, so neighbouring CTAs share A and B tiles in
// L2).  K in blocks of 32 (one 64-byte swizzle atom), 4 shared-memory stages
// of 48 KB.  Two TMEM accumulators of 256 columns: the epilogue of tile i
// (warps 2-5) overlaps the MMAs of tile i+1 (warp 1).
constexpr int BM = 128, BN = 256, BK = 32, STAGES = 4, GROUP_M = 8;
constexpr int A_TILE = BM * BK * 2;            // 8 KB
constexpr int B_TILE = BN * BK * 2;            // 16 KB
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr int EPI_BYTES = 4 * 32 * 33 * 4;     // per-warp 32 x 32 staging, padded
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EPI_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int NT = 192;
constexpr uint32_t ACC_COLS = 256, TMEM_COLS = 512;

struct EpiParams {
    float *C;
    int64_t M, N, ldc;
    float alpha, beta;
    int semantics;
    int num_kb;
    int tiles_m, tiles_n;
    int *err;
};

__device__ __forceinline__ void tile_coords(int t, int tiles_m, int tiles_n, int &tm, int &tn) {
    const int per_group = GROUP_M * tiles_n;
    const int g = t / per_group;
    const int first_m = g * GROUP_M;
    const int gm = min(GROUP_M, tiles_m - first_m);
    const int r = t - g * per_group;
    tm = first_m + r % gm;
    tn = r / gm;
}

__global__ void __launch_bounds__(NT, 1)
    bf16x3_gemm_kernel(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                       const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
                       EpiParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    float *epi = reinterpret_cast<float *>(smem + STAGES * STAGE_BYTES);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES + EPI_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;     // [2]
    uint64_t *acc_empty = acc_full + 2;      // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int num_tiles = p.tiles_m * p.tiles_n;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            ptx::mbar_init(&acc_full[b], 1);
            ptx::mbar_init(&acc_empty[b], 4);   // one arrive per epilogue warp
        }
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
            int kbg = 0;   // running k-block counter across tiles (stage / phase)
            bool go = true;
            for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
                int tm, tn;
                tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
                const int m0 = tm * BM, n0 = tn * BN;
                for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
                    const int s = kbg % STAGES;
                    if (kbg >= STAGES && !ptx::mbar_wait(&empty[s], ((kbg / STAGES) & 1) ^ 1, p.err, 1)) {
                        go = false;
                        break;
                    }
                    uint8_t *st = smem + s * STAGE_BYTES;
                    ptx::mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
                    ptx::tma_load_2d(st, &tmAh, &full[s], kb * BK, m0);
                    ptx::tma_load_2d(st + A_TILE, &tmAl, &full[s], kb * BK, m0);
                    ptx::tma_load_2d(st + 2 * A_TILE, &tmBh, &full[s], kb * BK, n0);
                    ptx::tma_load_2d(st + 2 * A_TILE + B_TILE, &tmBl, &full[s], kb * BK, n0);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, BN);
            int kbg = 0, it = 0;
            bool go = true;
            for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x, it++) {
                const int b = it & 1;
                if (it >= 2 && !ptx::mbar_wait(&acc_empty[b], ((it >> 1) & 1) ^ 1, p.err, 2)) break;
                ptx::tc_fence_after();
                const uint32_t acc = tmem + (uint32_t)(b * ACC_COLS);
                for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
                    const int s = kbg % STAGES;
                    if (!ptx::mbar_wait(&full[s], (kbg / STAGES) & 1, p.err, 3)) { go = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t st = ptx::smem_u32(smem + s * STAGE_BYTES);
                    const uint64_t ah = ptx::sdesc_kmajor_sw64(st);
                    const uint64_t al = ptx::sdesc_kmajor_sw64(st + A_TILE);
                    const uint64_t bh = ptx::sdesc_kmajor_sw64(st + 2 * A_TILE);
                    const uint64_t bl = ptx::sdesc_kmajor_sw64(st + 2 * A_TILE + B_TILE);
#pragma unroll
                    for (int k = 0; k < BK / 16; k++) {
                        // advance 16 BF16 = 32 bytes along K inside the 64-byte swizzle atom
                        const uint64_t dk = (uint64_t)((k * 32) >> 4);
                        ptx::umma_f16(acc, al + dk, bh + dk, idesc, (kb | k) != 0);
                        ptx::umma_f16(acc, ah + dk, bl + dk, idesc, 1);
                        ptx::umma_f16(acc, ah + dk, bh + dk, idesc, 1);
                    }
                    ptx::umma_commit(&empty[s]);
                }
                if (go) ptx::umma_commit(&acc_full[b]);
            }
        }
    } else {               // epilogue: warps 2..5 own TMEM lane quarters (warp % 4)
        const int q = warp % 4;
        float *stage = epi + q * 32 * 33;
        int it = 0;
        for (int t = blockIdx.x; t < num_tiles; t += gridDim.x, it++) {
            const int b = it & 1;
            if (!ptx::mbar_wait(&acc_full[b], (it >> 1) & 1, p.err, 4)) break;
            ptx::tc_fence_after();
            int tm, tn;
            tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
            const int64_t row0 = (int64_t)tm * BM + q * 32;
            const int64_t n0 = (int64_t)tn * BN;
            for (int c = 0; c < BN; c += 32) {
                uint32_t r[32];
                ptx::tmem_ld_32x32b_x32(tmem + (uint32_t)(b * ACC_COLS) + ((uint32_t)(q * 32) << 16) + (uint32_t)c,
                                        r);
                ptx::tmem_ld_wait();
                // thread `lane` holds row row0+lane, columns c..c+31: transpose through
                // shared memory so each store instruction writes one row contiguously
#pragma unroll
                for (int j = 0; j < 32; j++) stage[lane * 33 + j] = __uint_as_float(r[j]);
                __syncwarp();
                const int64_t col = n0 + c + lane;
                if (col < p.N) {
                    const int rows = (p.M - row0) < 32 ? (int)(p.M - row0) : 32;
                    if (p.semantics == GB_SEM_SCALAR_BETA || (p.semantics == GB_SEM_BLAS && p.beta == 0.f)) {
                        const float add = p.semantics == GB_SEM_SCALAR_BETA ? p.beta : 0.f;
                        for (int rr = 0; rr < rows; rr++)
                            p.C[(row0 + rr) * p.ldc + col] = p.alpha * stage[rr * 33 + lane] + add;
                    } else {
                        float cin[32];
#pragma unroll
                        for (int rr = 0; rr < 32; rr++)
                            cin[rr] = rr < rows ? p.C[(row0 + rr) * p.ldc + col] : 0.f;
#pragma unroll
                        for (int rr = 0; rr < 32; rr++) {
                            if (rr < rows) {
                                float v = p.alpha * stage[rr * 33 + lane];
                                v = p.semantics == GB_SEM_BLAS ? fmaf(p.beta, cin[rr], v) : cin[rr] + (v + p.beta);
                                p.C[(row0 + rr) * p.ldc + col] = v;
                            }
                        }
                    }
                }
                __syncwarp();
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&acc_empty[b]);
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
    const int64_t kp = ceil_div(g.K, 64) * 64;   // multiple of BK, zero-padded
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
    bool okm = make_tmap_bf16(&tAh, ah, kp, g.M, kp * 2, BK, BM, 64) &&
               make_tmap_bf16(&tAl, al, kp, g.M, kp * 2, BK, BM, 64) &&
               make_tmap_bf16(&tBh, bh, kp, g.N, kp * 2, BK, BN, 64) &&
               make_tmap_bf16(&tBl, bl, kp, g.N, kp * 2, BK, BN, 64);
    if (!okm) return set_status(GB_ERR_CUDA, "bf16x3: cuTensorMapEncodeTiled failed");

    static bool attr_set = false;
    if (!attr_set) {
        GB_CUDA_TRY(cudaFuncSetAttribute(bf16x3_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        attr_set = true;
    }
    const int tiles_m = (int)ceil_div(g.M, BM), tiles_n = (int)ceil_div(g.N, BN);
    EpiParams p{(float *)g.C, g.M, g.N, g.ldc, (float)g.alpha, (float)g.beta, g.semantics, (int)(kp / BK),
                tiles_m, tiles_n, err};
    const int tiles = tiles_m * tiles_n;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    bf16x3_gemm_kernel<<<grid, NT, SMEM_BYTES, g.stream>>>(tAh, tAl, tBh, tBl, p);
    GB_LAUNCH_CHECK("bf16x3_gemm_kernel");
    return ok();
}

}  // namespace gb
