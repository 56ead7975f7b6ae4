// skinny_tc.cu -- FP32 skinny GEMM with 8 < n <= 64 as 3xBF16 on tcgen05.
//
// Same problem as skinny.cu (irr_thinB / irr_shortA, the large operand X is
// rows x K, the small one W is K x n, C(r, j) at C[r*cs_r + j*cs_c]), for a
// small dimension where FP32 FFMA could no longer keep up with HBM: at n = 64
// the products need 8x the FFMA rate that streaming X at full bandwidth
// allows.  The products run on the tensor cores as
//     x_hi*w_hi + x_hi*w_lo + x_lo*w_hi      (BF16 pieces, FP32 accumulate)
// and X is split in flight, never written back to HBM:
//   * warp 0 (TMA) streams 128 x 32 FP32 tiles of X (row-major X as 128-byte
//     swizzled rows, K-major X as [32 k][128 rows]) and the matching BF16
//     tiles of W_hi / W_lo (W is split once per call by wsplit_kernel into
//     [NB][Kp] K-major pieces, a few hundred KB that stay in L2);
//   * warps 2-5 (one per TMEM lane quarter) each own 32 rows: a thread reads
//     its row's 32 values from shared memory, splits them and writes hi / lo
//     straight into tensor memory (tcgen05.st) -- the MMA reads A from TMEM,
//     so the split pieces never touch shared memory;
//   * warp 1 issues tcgen05.mma (M = 128, N = NB, K = 16, A from TMEM, B from
//     shared memory) into one of two TMEM accumulators of NB columns;
//   * warps 6-9 read the finished accumulator (tcgen05.ld) and apply
//     alpha / beta, or write split-K partials for skinny_reduce_kernel.
// Shared-memory traffic per X value is the TMA write and one read (8 bytes),
// well inside the SM's budget at full HBM rate.
#include <cuda.h>
#include <cuda_bf16.h>

#include "gb_common.cuh"
#include "sm100_ptx.cuh"

namespace gb {

bool make_tmap_f32(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                   uint32_t box_inner, uint32_t box_outer, bool sw128);
bool make_tmap_bf16(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                    uint32_t box_inner, uint32_t box_outer, int swizzle_bytes);

namespace {
namespace thin_tc {

constexpr int BM = 128, BK = 32, STAGES = 8, ASLOTS = 8, NT = 320;
constexpr uint32_t A_COL0 = 128;      // A slot i at TMEM columns 128 + 32 i (hi: +0..15, lo: +16..31)
constexpr uint32_t TMEM_COLS = 512;   // accumulators at columns [0, 2 NB)

template <int NB>
struct Cfg {
    static constexpr int XS = BM * BK * 4;   // 16 KB FP32 X tile
    static constexpr int WP = NB * BK * 2;   // one BF16 piece of W (NB rows of 64 bytes)
    static constexpr int STAGE = (XS + 2 * WP + 1023) / 1024 * 1024;
    static constexpr int SMEM = STAGES * STAGE + 1024 /*align*/ + 512 /*barriers*/;
};

struct TcParams {
    int64_t rows, K;
    int n, splits, kchunk_kb, rtiles;
    float *C; int64_t cs_r, cs_c;
    float alpha, beta;
    int semantics;
    float *part;
    int *err;
};

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) {
    return *reinterpret_cast<uint32_t *>(&v);
}

template <int NB, bool XCOLS>
__global__ void __launch_bounds__(NT, 1)
    thin_tc_kernel(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmwh,
                   const __grid_constant__ CUtensorMap tmwl, TcParams p) {
    using C = Cfg<NB>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * C::STAGE);
    uint64_t *empty = full + STAGES;
    uint64_t *aready = empty + STAGES;
    uint64_t *aempty = aready + ASLOTS;
    uint64_t *accf = aempty + ASLOTS;
    uint64_t *acce = accf + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acce + 2);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int nkb = (int)((p.K + BK - 1) / BK);
    const int units = p.rtiles * p.splits;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1 + 4);   // the MMA commit + the four converter warps
        }
        for (int a = 0; a < ASLOTS; a++) {
            ptx::mbar_init(&aready[a], 4);
            ptx::mbar_init(&aempty[a], 1);
        }
        for (int b = 0; b < 2; b++) {
            ptx::mbar_init(&accf[b], 1);
            ptx::mbar_init(&acce[b], 4);
        }
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&tmx);
        ptx::tma_prefetch_desc(&tmwh);
        ptx::tma_prefetch_desc(&tmwl);
    }
    if (warp == 1) ptx::tmem_alloc(tmem_slot, TMEM_COLS);
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {   // TMA producer
            int g = 0;
            bool go = true;
            for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
                const int rt = u / p.splits, sp = u - rt * p.splits;
                const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
                for (int kb = kb0; kb < kb1; kb++, g++) {
                    const int s = g % STAGES;
                    if (g >= STAGES && !ptx::mbar_wait(&empty[s], ((g / STAGES) & 1) ^ 1, p.err, 51)) {
                        go = false;
                        break;
                    }
                    uint8_t *st = smem + s * C::STAGE;
                    ptx::mbar_arrive_expect_tx(&full[s], C::XS + 2 * C::WP);
                    if (XCOLS) ptx::tma_load_2d(st, &tmx, &full[s], rt * BM, kb * BK);
                    else ptx::tma_load_2d(st, &tmx, &full[s], kb * BK, rt * BM);
                    ptx::tma_load_2d(st + C::XS, &tmwh, &full[s], kb * BK, 0);
                    ptx::tma_load_2d(st + C::XS + C::WP, &tmwl, &full[s], kb * BK, 0);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, NB);
            int g = 0, it = 0;
            bool go = true;
            for (int u = blockIdx.x; u < units && go; u += gridDim.x, it++) {
                const int sp = u % p.splits;
                const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
                const int b = it & 1;
                if (it >= 2 && !ptx::mbar_wait(&acce[b], ((it >> 1) & 1) ^ 1, p.err, 52)) break;
                ptx::tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(b * NB);
                for (int kb = kb0; kb < kb1; kb++, g++) {
                    const int s = g % STAGES, a = g % ASLOTS;
                    if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 53) ||
                        !ptx::mbar_wait(&aready[a], (g / ASLOTS) & 1, p.err, 54)) {
                        go = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const uint32_t st = ptx::smem_u32(smem + s * C::STAGE);
                    const uint64_t bh = ptx::sdesc_kmajor_sw64(st + C::XS);
                    const uint64_t bl = ptx::sdesc_kmajor_sw64(st + C::XS + C::WP);
                    const uint32_t ah = tmem + A_COL0 + (uint32_t)(a * 32), al = ah + 16u;
#pragma unroll
                    for (int kk = 0; kk < BK / 16; kk++) {
                        const uint64_t dk = (uint64_t)((kk * 32) >> 4);   // 16 BF16 = 32 bytes along K
                        const uint32_t ck = (uint32_t)(kk * 8);           // 16 BF16 = 8 TMEM columns
                        ptx::umma_f16_ta(d, al + ck, bh + dk, idesc, (kb != kb0 || kk != 0) ? 1u : 0u);
                        ptx::umma_f16_ta(d, ah + ck, bl + dk, idesc, 1u);
                        ptx::umma_f16_ta(d, ah + ck, bh + dk, idesc, 1u);
                    }
                    ptx::umma_commit(&empty[s]);
                    ptx::umma_commit(&aempty[a]);
                }
                if (go) ptx::umma_commit(&accf[b]);
            }
        }
    } else if (warp < 6) {   // converters: thread = row q*32 + lane of the tile
        const int q = warp % 4, r = q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int g = 0;
        bool go = true;
        for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
            const int sp = u % p.splits;
            const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
            for (int kb = kb0; kb < kb1; kb++, g++) {
                const int s = g % STAGES, a = g % ASLOTS;
                if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 55) ||
                    (g >= ASLOTS && !ptx::mbar_wait(&aempty[a], ((g / ASLOTS) & 1) ^ 1, p.err, 56))) {
                    go = false;
                    break;
                }
                ptx::tc_fence_after();
                const uint8_t *st = smem + s * C::STAGE;
                float x[BK];
                if (XCOLS) {
                    const float *xs = reinterpret_cast<const float *>(st);
#pragma unroll
                    for (int k = 0; k < BK; k++) x[k] = xs[k * BM + r];
                } else {
                    const uint8_t *row = st + r * 128;
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        const float4 v = *reinterpret_cast<const float4 *>(row + ((c ^ (r & 7)) << 4));
                        x[4 * c] = v.x; x[4 * c + 1] = v.y; x[4 * c + 2] = v.z; x[4 * c + 3] = v.w;
                    }
                }
                uint32_t pk[32];
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const __nv_bfloat162 h = __floats2bfloat162_rn(x[2 * i], x[2 * i + 1]);
                    const float2 hf = __bfloat1622float2(h);
                    const __nv_bfloat162 l = __floats2bfloat162_rn(x[2 * i] - hf.x, x[2 * i + 1] - hf.y);
                    pk[i] = bf16x2_bits(h);
                    pk[16 + i] = bf16x2_bits(l);
                }
                ptx::tmem_st_32x32b_x32(tmem + lane_off + A_COL0 + (uint32_t)(a * 32), pk);
                ptx::tmem_st_wait();
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) {
                    ptx::mbar_arrive(&aready[a]);
                    ptx::mbar_arrive(&empty[s]);
                }
            }
        }
    } else {                 // epilogue: thread = row q*32 + lane of the tile
        const int q = warp % 4;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int it = 0;
        for (int u = blockIdx.x; u < units; u += gridDim.x, it++) {
            const int rt = u / p.splits, sp = u - rt * p.splits;
            const int b = it & 1;
            if (!ptx::mbar_wait(&accf[b], (it >> 1) & 1, p.err, 57)) break;
            ptx::tc_fence_after();
            float acc[NB];
#pragma unroll
            for (int c = 0; c < NB; c += 16) {
                uint32_t v[16];
                ptx::tmem_ld_32x32b_x16(tmem + lane_off + (uint32_t)(b * NB + c), v);
                ptx::tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 16; j++) acc[c + j] = __uint_as_float(v[j]);
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&acce[b]);
            const int64_t row = (int64_t)rt * BM + q * 32 + lane;
            if (row >= p.rows) continue;
            if (p.splits > 1) {
                float *pp = p.part + ((int64_t)sp * p.rows + row) * NB;
#pragma unroll
                for (int j = 0; j < NB; j += 4)
                    *reinterpret_cast<float4 *>(pp + j) = make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]);
                continue;
            }
            float *cr = p.C + row * p.cs_r;
#pragma unroll
            for (int j = 0; j < NB; j++) {
                if (j >= p.n) break;
                float *cp = cr + (int64_t)j * p.cs_c;
                float v = p.alpha * acc[j];
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

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// W (logical K x n; tw: stored n x K) -> hi / lo BF16 pieces [NB][kp], K-major,
// zero beyond n and K.
__global__ void wsplit_kernel(const float *__restrict__ W, int64_t ldw, int tw, int n, int64_t K, int64_t kp, int nb,
                              __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ lo) {
    const int64_t total = (int64_t)nb * kp;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / kp, k = e - j * kp;
        float v = 0.f;
        if (j < n && k < K) v = tw ? W[j * ldw + k] : W[k * ldw + j];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[e] = h;
        lo[e] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

template <int NB, bool XCOLS>
gb_status launch_nb(const ThinTcArgs &a, const CUtensorMap &tx, const CUtensorMap &twh, const CUtensorMap &twl,
                    const TcParams &tp, int grid) {
    static bool attr = false;
    if (!attr) {
        GB_CUDA_TRY(cudaFuncSetAttribute(thin_tc_kernel<NB, XCOLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Cfg<NB>::SMEM));
        attr = true;
    }
    thin_tc_kernel<NB, XCOLS><<<grid, NT, Cfg<NB>::SMEM, a.stream>>>(tx, twh, twl, tp);
    GB_LAUNCH_CHECK("thin_tc_kernel");
    return ok();
}

}  // namespace thin_tc
}  // namespace

size_t thin_tc_wpieces_bytes(int nb, int64_t K) {
    const int64_t kp = ceil_div(K, thin_tc::BK) * thin_tc::BK;
    return (size_t)2 * nb * kp * 2;
}

gb_status launch_thin_tc(const ThinTcArgs &a) {
    using namespace thin_tc;
    const int64_t kp = ceil_div(a.K, BK) * BK;
    __nv_bfloat16 *wh = (__nv_bfloat16 *)a.wpieces, *wl = wh + (size_t)a.nb * kp;
    {
        const int64_t total = (int64_t)a.nb * kp;
        const int blocks = (int)(ceil_div(total, 256) < 2 * sm_count() ? ceil_div(total, 256) : 2 * sm_count());
        wsplit_kernel<<<blocks, 256, 0, a.stream>>>(a.W, a.ldw, a.tw, a.n, a.K, kp, a.nb, wh, wl);
        GB_LAUNCH_CHECK("wsplit_kernel");
    }
    CUtensorMap tx, twh, twl;
    bool okm = a.tx ? make_tmap_f32(&tx, a.X, (uint64_t)a.rows, (uint64_t)a.K, (uint64_t)a.ldx * 4, BM, BK, false)
                    : make_tmap_f32(&tx, a.X, (uint64_t)a.K, (uint64_t)a.rows, (uint64_t)a.ldx * 4, BK, BM, true);
    okm = okm && make_tmap_bf16(&twh, wh, (uint64_t)kp, (uint64_t)a.nb, (uint64_t)kp * 2, BK, (uint32_t)a.nb, 64);
    okm = okm && make_tmap_bf16(&twl, wl, (uint64_t)kp, (uint64_t)a.nb, (uint64_t)kp * 2, BK, (uint32_t)a.nb, 64);
    if (!okm) return set_status(GB_ERR_CUDA, "skinny: cuTensorMapEncodeTiled failed");
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "skinny: no device error word");
    TcParams tp{a.rows, a.K, a.n, a.splits, (int)(a.kchunk / BK), (int)a.rtiles, a.C, a.cs_r, a.cs_c,
                a.alpha, a.beta, a.semantics, a.part, err};
    const int64_t units = a.rtiles * a.splits;
    const int grid = (int)(units < sm_count() ? units : sm_count());
    switch (a.nb * 2 + (a.tx ? 1 : 0)) {
        case 32: return launch_nb<16, false>(a, tx, twh, twl, tp, grid);
        case 33: return launch_nb<16, true>(a, tx, twh, twl, tp, grid);
        case 64: return launch_nb<32, false>(a, tx, twh, twl, tp, grid);
        case 65: return launch_nb<32, true>(a, tx, twh, twl, tp, grid);
        case 128: return launch_nb<64, false>(a, tx, twh, twl, tp, grid);
        case 129: return launch_nb<64, true>(a, tx, twh, twl, tp, grid);
        default: return set_status(GB_ERR_UNSUPPORTED, "skinny: no tensor-core tile for n = %d", a.n);
    }
}

}  // namespace gb
