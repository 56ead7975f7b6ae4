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
#include <stdlib.h>
#include <string.h>

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

// 2-D FP32 tensor [outer][inner], box box_inner x box_outer, no swizzle or
// 128-byte swizzle (box_inner * 4 must then be 128).
bool make_tmap_f32(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                   uint32_t box_inner, uint32_t box_outer, bool sw128) {
    PFN_encodeTiled enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, sw128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// 2-D FP64 tensor [outer][inner], box box_inner x box_outer, no swizzle or
// 128-byte swizzle (box_inner * 8 must then be 128).
bool make_tmap_f64(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                   uint32_t box_inner, uint32_t box_outer, bool sw128) {
    PFN_encodeTiled enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, sw128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

namespace {

// ------------------------------------------------------------------ split
// out_hi/out_lo(/out_lo2): rows x kp (K-major).  Source element (r, k):
// trans ? X[k*ldx + r] : X[r*ldx + k].  32x32 tiles through shared memory
// so both the read and the write are coalesced in either layout.  With
// out_lo2 the value is cut in three BF16 pieces (hi, mid, lo: 24 bits).
__global__ void __launch_bounds__(256) split_kernel(const float *__restrict__ X, int64_t ldx, int trans, int64_t rows,
                                                    int64_t K, int64_t kp, __nv_bfloat16 *__restrict__ out_hi,
                                                    __nv_bfloat16 *__restrict__ out_lo,
                                                    __nv_bfloat16 *__restrict__ out_lo2) {
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
            const float rem = x - __bfloat162float(h);   // exact
            __nv_bfloat16 l = __float2bfloat16_rn(rem);
            out_hi[r * kp + k] = h;
            out_lo[r * kp + k] = l;
            if (out_lo2) out_lo2[r * kp + k] = __float2bfloat16_rn(rem - __bfloat162float(l));
        }
    }
    // launched to overlap the previous call's GEMM (programmatic stream serialization): one
    // thread keeps the grid from completing before that grid has, so the stream order of the
    // GEMM that follows is unchanged
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) ptx::pdl_wait();
}

// Vectorised split of both operands in one launch (16-byte aligned sources
// with leading dimensions a multiple of 4).  A CTA converts a 64 x 64 block
// of (row, k): a K-contiguous source is read and written 4 values at a time
// straight from registers; a row-contiguous source is read 4 rows at a time
// into shared memory and written 4 k at a time.  Same values as
// split_kernel, about two-thirds of its time at the 4096^2 operands.
struct SplitOp {
    const float *X;
    int64_t ldx, rows, tiles_k, tiles;
    int trans;                      // source element (r, k) at X[k*ldx + r]
    __nv_bfloat16 *out[3];
};
struct SplitArgs {
    SplitOp op[2];
    int64_t K, kp;
    int np;
};

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

__device__ __forceinline__ void split_store4(const SplitArgs &a, const SplitOp &o, int64_t r, int64_t k,
                                             const float (&v)[4]) {
    __nv_bfloat16 h[4], l[4], l2[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        h[q] = __float2bfloat16_rn(v[q]);
        const float rem = v[q] - __bfloat162float(h[q]);   // exact
        l[q] = __float2bfloat16_rn(rem);
        l2[q] = __float2bfloat16_rn(rem - __bfloat162float(l[q]));
    }
    const int64_t off = r * a.kp + k;
    *reinterpret_cast<uint2 *>(o.out[0] + off) = make_uint2(pack2(h[0], h[1]), pack2(h[2], h[3]));
    *reinterpret_cast<uint2 *>(o.out[1] + off) = make_uint2(pack2(l[0], l[1]), pack2(l[2], l[3]));
    if (a.np == 3)
        *reinterpret_cast<uint2 *>(o.out[2] + off) = make_uint2(pack2(l2[0], l2[1]), pack2(l2[2], l2[3]));
}

__global__ void __launch_bounds__(256) split_vec_kernel(const __grid_constant__ SplitArgs a) {
    __shared__ float tile[64][65];
    int64_t b = blockIdx.x;
    const int w = b < a.op[0].tiles ? 0 : 1;
    if (w) b -= a.op[0].tiles;
    const SplitOp &o = a.op[w];
    const int64_t r0 = (b / o.tiles_k) * 64, k0 = (b % o.tiles_k) * 64;
    const int t = threadIdx.x, c4 = 4 * (t % 16), rl = t / 16;
    if (!o.trans) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int64_t r = r0 + rl + 16 * i, k = k0 + c4;
            if (r >= o.rows) continue;
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            const float *src = o.X + r * o.ldx + k;
            if (k + 3 < a.K) {
                const float4 x = __ldg(reinterpret_cast<const float4 *>(src));
                v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (k + q < a.K) v[q] = src[q];
            }
            split_store4(a, o, r, k, v);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) ptx::pdl_wait();   // as split_kernel
        return;
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {   // tile[k][r], 4 consecutive r per load
        const int kl = rl + 16 * i;
        const int64_t k = k0 + kl, r = r0 + c4;
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k < a.K) {
            const float *src = o.X + k * o.ldx + r;
            if (r + 3 < o.rows) {
                x = __ldg(reinterpret_cast<const float4 *>(src));
            } else {
                if (r < o.rows) x.x = src[0];
                if (r + 1 < o.rows) x.y = src[1];
                if (r + 2 < o.rows) x.z = src[2];
            }
        }
        tile[kl][c4] = x.x; tile[kl][c4 + 1] = x.y; tile[kl][c4 + 2] = x.z; tile[kl][c4 + 3] = x.w;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int rr = rl + 16 * i;
        const int64_t r = r0 + rr;
        if (r >= o.rows) continue;
        const float v[4] = {tile[c4][rr], tile[c4 + 1][rr], tile[c4 + 2][rr], tile[c4 + 3][rr]};
        split_store4(a, o, r, k0 + c4, v);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ptx::pdl_wait();   // as split_kernel
}

// ------------------------------------------------------------------- gemm
// Persistent: one CTA per SM walks the 128 x BN C tiles in a grouped order
// (GROUP_M tile rows at a time, so neighbouring CTAs share A and B tiles in
// L2).  K in blocks of 32 (one 64-byte swizzle atom), 4 shared-memory stages
// of 48 KB holding NP BF16 pieces of the A and B tiles (NP = 2: hi, lo with
// BN = 256; NP = 3: hi, mid, lo with BN = 128).  Two TMEM accumulators of BN
// columns: the epilogue of tile i (warps 2-5) overlaps the MMAs of tile i+1
// (warp 1).
constexpr int BM = 128, BK = 32, STAGES = 4, GROUP_M = 8;
constexpr int A_TILE = BM * BK * 2;            // 8 KB
constexpr int EPI_BYTES = 4 * 32 * 33 * 4;     // per-warp 32 x 32 staging, padded
constexpr int NT = 192;

template <int NP, int BN>
struct TwoPass {
    static constexpr int B_TILE = BN * BK * 2;
    static constexpr int STAGE_BYTES = NP * A_TILE + NP * B_TILE;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EPI_BYTES + 1024 /*align*/ + 256 /*barriers*/;
    static constexpr uint32_t ACC_COLS = BN, TMEM_COLS = 2 * BN;
};

// tensor maps of the A and B pieces (hi, lo[, lo2])
struct PieceMaps {
    CUtensorMap a[3], b[3];
    CUtensorMap bh[3];   // B pieces with 128-row boxes (half tiles of the tail wave)
};

struct EpiParams {
    float *C;
    int64_t M, N, ldc;
    float alpha, beta;
    int semantics;
    int num_kb;
    int tiles_m, tiles_n;
    int *err;
    int chunk_kb;    // k-blocks per accumulator chunk (folding form)
    // Stream-K tail: tiles [0, dp_tiles) go whole to CTAs in turn; the K
    // iterations of tiles [dp_tiles, tiles) are split evenly over the grid, so
    // a tile there may be computed in two parts (by CTAs b and b + 1): each
    // part's raw accumulator goes to sk_part[2b + half], and the second CTA to
    // finish (sk_cnt[b]) adds the two in order and writes C.
    int dp_tiles;
    float *sk_part;
    int *sk_cnt;
    // Half-tile tail: tiles [half_start, tiles) (a last wave at most half
    // full) run as two 128-column halves on different CTAs, so the wave takes
    // half a tile time.
    int half_start;
};

// Work items of one CTA: (tile, k-blocks [kb0, kb1), half: -1 whole tile,
// 0 / 1 the left / right 128 columns).
struct WorkIt {
    int i;
    int64_t pos, end;   // stream-K position / end in (tile - dp_tiles) * num_kb + kb
};

__device__ __forceinline__ bool next_item(const EpiParams &p, int num_tiles, WorkIt &w, int &tile, int &kb0,
                                          int &kb1, int &half) {
    half = -1;
    if (p.half_start < num_tiles) {   // whole tiles, then the tail in halves
        const int t = blockIdx.x + w.i * gridDim.x;
        w.i++;
        kb0 = 0; kb1 = p.num_kb;
        if (t < p.half_start) { tile = t; return true; }
        const int h = t - p.half_start;
        if (h >= 2 * (num_tiles - p.half_start)) return false;
        tile = p.half_start + h / 2;
        half = h & 1;
        return true;
    }
    if (w.pos < 0) {
        const int t = blockIdx.x + w.i * gridDim.x;
        if (t < p.dp_tiles) {
            tile = t; kb0 = 0; kb1 = p.num_kb; w.i++;
            return true;
        }
        const int64_t W = (int64_t)(num_tiles - p.dp_tiles) * p.num_kb;
        w.pos = W * blockIdx.x / gridDim.x;
        w.end = W * (blockIdx.x + 1) / gridDim.x;
    }
    if (w.pos >= w.end) return false;
    if (blockIdx.x & 1) {
        // odd CTAs walk their range backwards, so both parts of every split
        // tile are computed at the same time (by the end of two neighbours'
        // walks or by their start) and share its operand tiles in L2
        const int st = (int)((w.end - 1) / p.num_kb);
        const int64_t t0 = (int64_t)st * p.num_kb;
        const int64_t s0 = w.pos > t0 ? w.pos : t0;
        kb0 = (int)(s0 - t0);
        kb1 = (int)(w.end - t0);
        tile = p.dp_tiles + st;
        w.end = s0;
        return true;
    }
    const int st = (int)(w.pos / p.num_kb);
    kb0 = (int)(w.pos - (int64_t)st * p.num_kb);
    const int64_t left = w.end - w.pos;
    kb1 = left < p.num_kb - kb0 ? kb0 + (int)left : p.num_kb;
    tile = p.dp_tiles + st;
    w.pos += kb1 - kb0;
    return true;
}

__device__ __forceinline__ void tile_coords(int t, int tiles_m, int tiles_n, int &tm, int &tn) {
    const int per_group = GROUP_M * tiles_n;
    const int g = t / per_group;
    const int first_m = g * GROUP_M;
    const int gm = min(GROUP_M, tiles_m - first_m);
    const int r = t - g * per_group;
    tm = first_m + r % gm;
    tn = r / gm;
}

// FOLD: the tensor cores add each MMA into the FP32 accumulator with an
// error of about one unit in the last place of the accumulator, so over a
// long K the error grows with the number of MMAs and with the size of the
// running sum.  With FOLD the accumulator is restarted every chunk_kb
// k-blocks (chunk_kb * 32 values of K) and the epilogue warps add each chunk
// into an FP32 running total held in registers (round-to-nearest), and the
// most significant product hi*hi is accumulated apart from the small
// cross products, so only the hi*hi MMAs add into a large accumulator.
// TMEM: two chunk buffers of 256 columns (hi*hi at +0, the rest at +128),
// BN = 128; the MMAs of chunk c+1 overlap the fold of chunk c.
template <int NP, int BN, bool FOLD>
__global__ void __launch_bounds__(NT, 1) bf16x3_gemm_kernel(const __grid_constant__ PieceMaps maps, EpiParams p) {
    // the next call's split pass may start beside this grid (it writes the other workspace half)
    if (threadIdx.x == 0) ptx::pdl_launch_dependents();
    using CF = TwoPass<NP, BN>;
    static_assert(!FOLD || BN == 128, "the folding form keeps a 128-column total per thread");
    constexpr int B_TILE = CF::B_TILE, STAGE_BYTES = CF::STAGE_BYTES;
    constexpr uint32_t ACC_COLS = FOLD ? 256 : CF::ACC_COLS, TMEM_COLS = FOLD ? 512 : CF::TMEM_COLS;
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
    const int chunk_kb = FOLD ? p.chunk_kb : p.num_kb;

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
        for (int i = 0; i < NP; i++) {
            ptx::tma_prefetch_desc(&maps.a[i]);
            ptx::tma_prefetch_desc(&maps.b[i]);
        }
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
            WorkIt wi{0, -1, 0};
            int t, kbA, kbB, half;
            while (go && next_item(p, num_tiles, wi, t, kbA, kbB, half)) {
                int tm, tn;
                tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
                const int m0 = tm * BM, n0 = tn * BN + (half > 0 ? BN / 2 : 0);
                const uint32_t bytes = half < 0 ? STAGE_BYTES : NP * A_TILE + NP * (B_TILE / 2);
                for (int kb = kbA; kb < kbB; kb++, kbg++) {
                    const int s = kbg % STAGES;
                    if (kbg >= STAGES && !ptx::mbar_wait(&empty[s], ((kbg / STAGES) & 1) ^ 1, p.err, 1)) {
                        go = false;
                        break;
                    }
                    uint8_t *st = smem + s * STAGE_BYTES;
                    ptx::mbar_arrive_expect_tx(&full[s], bytes);
#pragma unroll
                    for (int i = 0; i < NP; i++) {
                        ptx::tma_load_2d(st + i * A_TILE, &maps.a[i], &full[s], kb * BK, m0);
                        ptx::tma_load_2d(st + NP * A_TILE + i * B_TILE, half < 0 ? &maps.b[i] : &maps.bh[i],
                                         &full[s], kb * BK, n0);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, BN);
            int kbg = 0, ch = 0;   // running k-block and accumulator-chunk counters
            (void)B_TILE;
            bool go = true;
            constexpr uint32_t idesc_half = ptx::idesc_bf16_f32(BM, BN / 2);
            WorkIt wi{0, -1, 0};
            int t, kbA, kbB, half;
            while (go && next_item(p, num_tiles, wi, t, kbA, kbB, half)) {
                const uint32_t id = half < 0 ? idesc : idesc_half;
                const int nch = (kbB - kbA + chunk_kb - 1) / chunk_kb;
                for (int c = 0; c < nch && go; c++, ch++) {
                    const int b = ch & 1;
                    if (ch >= 2 && !ptx::mbar_wait(&acc_empty[b], ((ch >> 1) & 1) ^ 1, p.err, 2)) {
                        go = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const uint32_t acc = tmem + (uint32_t)(b * ACC_COLS);
                    const uint32_t acc_lo = FOLD ? acc + 128u : acc;   // cross products
                    const int kbc = kbA + c * chunk_kb;
                    const int kb1 = kbc + chunk_kb < kbB ? kbc + chunk_kb : kbB;
                    for (int kb = kbc; kb < kb1; kb++, kbg++) {
                        const int s = kbg % STAGES;
                        if (!ptx::mbar_wait(&full[s], (kbg / STAGES) & 1, p.err, 3)) { go = false; break; }
                        ptx::tc_fence_after();
                        const uint32_t st = ptx::smem_u32(smem + s * STAGE_BYTES);
                        uint64_t ad[NP], bd[NP];
#pragma unroll
                        for (int i = 0; i < NP; i++) {
                            ad[i] = ptx::sdesc_kmajor_sw64(st + i * A_TILE);
                            bd[i] = ptx::sdesc_kmajor_sw64(st + NP * A_TILE + i * B_TILE);
                        }
                        const bool first = kb == kbc;
#pragma unroll
                        for (int k = 0; k < BK / 16; k++) {
                            // advance 16 BF16 = 32 bytes along K inside the 64-byte swizzle atom
                            const uint64_t dk = (uint64_t)((k * 32) >> 4);
                            // piece products (i, j) with i + j < NP, least significant first
#pragma unroll
                            for (int d = NP - 1; d >= 0; d--)
#pragma unroll
                                for (int i = d; i >= 0; i--) {
                                    const bool lead = FOLD ? (d == NP - 1 && i == d) || d == 0 : d == NP - 1 && i == d;
                                    ptx::umma_f16(d == 0 ? acc : acc_lo, ad[i] + dk, bd[d - i] + dk, id,
                                                  !(first && k == 0 && lead));
                                }
                        }
                        ptx::umma_commit(&empty[s]);
                    }
                    if (go) ptx::umma_commit(&acc_full[b]);
                }
            }
        }
    } else {               // epilogue: warps 2..5 own TMEM lane quarters (warp % 4)
        const int q = warp % 4;
        float *stage = epi + q * 32 * 33;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int ch = 0;
        float total[FOLD ? BN : 1];
        bool go = true;
        __shared__ int sk_last;
        WorkIt wi{0, -1, 0};
        int t, kbA, kbB, half;
        while (go && next_item(p, num_tiles, wi, t, kbA, kbB, half)) {
            int tm, tn;
            tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
            const int64_t row0 = (int64_t)tm * BM + q * 32;
            const int64_t n0 = (int64_t)tn * BN + (half > 0 ? BN / 2 : 0);
            const int ncols = half < 0 ? BN : BN / 2;
            // a stream-K part: raw accumulator to its slot, C written by the second finisher
            const bool part = !FOLD && (kbA != 0 || kbB != p.num_kb);
            const int sk_b = kbA == 0 ? (int)blockIdx.x : (int)blockIdx.x - 1;
            float *slot = part ? p.sk_part + ((size_t)sk_b * 2 + (kbA == 0 ? 0 : 1)) * (BM * BN) : nullptr;
            uint32_t accb = 0;
            if (FOLD) {
#pragma unroll
                for (int j = 0; j < (FOLD ? BN : 1); j++) total[j] = 0.f;
                for (int c = 0; c < (kbB - kbA + chunk_kb - 1) / chunk_kb; c++, ch++) {
                    const int b = ch & 1;
                    if (!ptx::mbar_wait(&acc_full[b], (ch >> 1) & 1, p.err, 4)) { go = false; break; }
                    ptx::tc_fence_after();
#pragma unroll
                    for (int g = 0; g < (FOLD ? BN : 32) / 32; g++) {
                        uint32_t rh[32], rl[32];
                        const uint32_t a = tmem + (uint32_t)(b * ACC_COLS) + lane_off + (uint32_t)(g * 32);
                        ptx::tmem_ld_32x32b_x32(a, rh);
                        ptx::tmem_ld_32x32b_x32(a + 128u, rl);
                        ptx::tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 32; j++)
                            total[g * 32 + j] += __uint_as_float(rh[j]) + __uint_as_float(rl[j]);
                    }
                    ptx::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) ptx::mbar_arrive(&acc_empty[b]);
                }
                if (!go) break;
            } else {
                const int b = ch & 1;
                if (!ptx::mbar_wait(&acc_full[b], (ch >> 1) & 1, p.err, 4)) break;
                ptx::tc_fence_after();
                accb = (uint32_t)(b * ACC_COLS);
            }
#pragma unroll
            for (int c = 0; c < BN; c += 32) {
                if (c >= ncols) break;
                // thread `lane` holds row row0+lane, columns c..c+31: transpose through
                // shared memory so each store instruction writes one row contiguously
                if (FOLD) {
#pragma unroll
                    for (int j = 0; j < 32; j++) stage[lane * 33 + j] = total[(FOLD ? c : 0) + j];
                } else {
                    uint32_t r[32];
                    ptx::tmem_ld_32x32b_x32(tmem + accb + lane_off + (uint32_t)c, r);
                    ptx::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; j++) stage[lane * 33 + j] = __uint_as_float(r[j]);
                }
                __syncwarp();
                if (part) {   // raw values, tile-local layout [row][col]
#pragma unroll
                    for (int rr = 0; rr < 32; rr++) slot[(q * 32 + rr) * BN + c + lane] = stage[rr * 33 + lane];
                    __syncwarp();
                    continue;
                }
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
            if (!FOLD) {
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&acc_empty[ch & 1]);
                ch++;
            }
            if (part) {
                __threadfence();                                  // this part is visible GPU-wide ...
                asm volatile("bar.sync 1, 128;" ::: "memory");   // ... for all four epilogue warps
                if (warp == 2 && lane == 0) {
                    const int old = atomicAdd(&p.sk_cnt[sk_b], 1);
                    if (old == 1) p.sk_cnt[sk_b] = 0;            // both parts done: reset for the next call
                    sk_last = old == 1;
                    __threadfence();
                }
                asm volatile("bar.sync 1, 128;" ::: "memory");
                if (sk_last) {   // left part + right part, in that order, then the epilogue
                    const float *p0 = p.sk_part + (size_t)sk_b * 2 * (BM * BN), *p1 = p0 + BM * BN;
                    const int rows = (p.M - row0) < 32 ? (int)(p.M - row0) : 32;
                    const bool read_c = p.semantics == GB_SEM_ACCUM_SCALAR_BETA ||
                                        (p.semantics == GB_SEM_BLAS && p.beta != 0.f);
                    for (int c = 0; c < BN; c += 32) {
                        const int64_t col = n0 + c + lane;
                        if (col >= p.N) continue;
                        // all 32 rows' loads in flight before any use
                        float v[32], cin[32];
#pragma unroll
                        for (int rr = 0; rr < 32; rr++) {
                            const int e = (q * 32 + rr) * BN + c + lane;
                            v[rr] = rr < rows ? __ldcg(p0 + e) + __ldcg(p1 + e) : 0.f;
                            cin[rr] = (read_c && rr < rows) ? p.C[(row0 + rr) * p.ldc + col] : 0.f;
                        }
#pragma unroll
                        for (int rr = 0; rr < 32; rr++) {
                            if (rr >= rows) break;
                            float x = p.alpha * v[rr];
                            if (p.semantics == GB_SEM_BLAS) x = p.beta != 0.f ? fmaf(p.beta, cin[rr], x) : x;
                            else if (p.semantics == GB_SEM_SCALAR_BETA) x = x + p.beta;
                            else x = cin[rr] + (x + p.beta);
                            p.C[(row0 + rr) * p.ldc + col] = x;
                        }
                    }
                }
                asm volatile("bar.sync 1, 128;" ::: "memory");   // sk_last is reused by the next part
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


// ============================================================ fused split
// The same 3xBF16 product without a separate split pass: TMA brings FP32
// tiles of op(A) (128 x 32) and op(B)^T (BN x 32) straight from the caller's
// matrices in whichever layout they are stored; 8 converter warps split each
// value into hi/lo BF16 and write them in the 64-byte-swizzled K-major layout
// the UMMA descriptors read (then fence the async proxy); the MMA and
// epilogue warps are those of the two-kernel form.  Roles: warp 0 TMA,
// warp 1 MMA, warps 2-5 epilogue, warps 6-13 converters.
namespace fused {

constexpr int BM = 128, BK = 32, GROUP_M = 8, NT = 448, NCONV = 8;

template <int BN>
struct Cfg {
    static constexpr int A32 = BM * BK * 4;                 // FP32 staging (16 KB)
    static constexpr int B32 = BN * BK * 4;
    static constexpr int ABF = BM * BK * 2;                 // one BF16 tile (8 KB)
    static constexpr int BBF = BN * BK * 2;
    static constexpr int STAGE32 = A32 + B32;
    static constexpr int STAGEBF = 2 * ABF + 2 * BBF;
    static constexpr int STAGES = (200 * 1024) / (STAGE32 + STAGEBF) >= 4 ? 4
                                  : (200 * 1024) / (STAGE32 + STAGEBF);
    static constexpr int EPI = 4 * 32 * 33 * 4;
    static constexpr int SMEM = STAGES * (STAGE32 + STAGEBF) + EPI + 1024 + 512;
    static constexpr uint32_t TMEM_COLS = 2 * BN;
};

struct Params {
    float *C;
    int64_t M, N, ldc;
    float alpha, beta;
    int semantics;
    int num_kb;
    int tiles_m, tiles_n;
    int a_kmajor, b_kmajor;      // FP32 staging layout of op(A) / op(B)^T
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

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}

// Split one 8-value K chunk of row r into the hi and lo BF16 tiles
// (64-byte swizzle: 16-byte chunk c of row r sits at chunk c ^ ((r % 8) / 2)).
__device__ __forceinline__ void split_store(const float (&v)[8], uint8_t *hi, uint8_t *lo, int r, int c) {
    float h[8], l[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        h[j] = __bfloat162float(__float2bfloat16_rn(v[j]));
        l[j] = v[j] - h[j];
    }
    const uint32_t off = (uint32_t)(r >> 3) * 512u + (uint32_t)(r & 7) * 64u + (uint32_t)((c ^ ((r & 7) >> 1)) << 4);
    *reinterpret_cast<uint4 *>(hi + off) =
        make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]), pack_bf16(h[6], h[7]));
    *reinterpret_cast<uint4 *>(lo + off) =
        make_uint4(pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]), pack_bf16(l[6], l[7]));
}

// Convert a ROWS x 32 FP32 staging tile into hi/lo BF16 tiles.  K-major
// staging is TMA-swizzled (128-byte rows, 16-byte piece p of row r at
// p ^ (r % 8)); MN-major staging is [32][ROWS] plain.
template <int ROWS>
__device__ __forceinline__ void convert_tile(const uint8_t *src, bool kmajor, uint8_t *hi, uint8_t *lo, int ctid) {
    constexpr int CHUNKS = ROWS * (BK / 8);
    for (int q = ctid; q < CHUNKS; q += NCONV * 32) {
        float v[8];
        int r, c;
        if (kmajor) {
            r = q >> 2;
            c = q & 3;
            const uint8_t *row = src + (r >> 3) * 1024 + (r & 7) * 128;
            const float4 a = *reinterpret_cast<const float4 *>(row + (((2 * c) ^ (r & 7)) << 4));
            const float4 b = *reinterpret_cast<const float4 *>(row + (((2 * c + 1) ^ (r & 7)) << 4));
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
            v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        } else {
            c = q / ROWS;
            r = q - c * ROWS;
            const float *col = reinterpret_cast<const float *>(src) + (c * 8) * ROWS + r;
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = col[j * ROWS];
        }
        split_store(v, hi, lo, r, c);
    }
}

template <int BN>
__global__ void __launch_bounds__(NT, 1)
    bf16x3_fused_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, Params p) {
    using C = Cfg<BN>;
    constexpr int S = C::STAGES;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *st32 = smem;                                  // S x (A32 + B32)
    uint8_t *stbf = smem + S * C::STAGE32;                 // S x (Ahi, Alo, Bhi, Blo)
    float *epi = reinterpret_cast<float *>(stbf + S * C::STAGEBF);
    uint64_t *f32_full = reinterpret_cast<uint64_t *>(reinterpret_cast<uint8_t *>(epi) + C::EPI);
    uint64_t *f32_empty = f32_full + S;
    uint64_t *bf_full = f32_empty + S;
    uint64_t *bf_empty = bf_full + S;
    uint64_t *acc_full = bf_empty + S;
    uint64_t *acc_empty = acc_full + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int num_tiles = p.tiles_m * p.tiles_n;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            ptx::mbar_init(&f32_full[s], 1);
            ptx::mbar_init(&f32_empty[s], NCONV);
            ptx::mbar_init(&bf_full[s], NCONV);
            ptx::mbar_init(&bf_empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            ptx::mbar_init(&acc_full[b], 1);
            ptx::mbar_init(&acc_empty[b], 4);
        }
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&tmA);
        ptx::tma_prefetch_desc(&tmB);
    }
    if (warp == 1) ptx::tmem_alloc(tmem_slot, C::TMEM_COLS);
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {   // TMA producer: FP32 tiles in their stored layout
            int kbg = 0;
            bool go = true;
            for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
                int tm, tn;
                tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
                const int m0 = tm * BM, n0 = tn * BN;
                for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
                    const int s = kbg % S;
                    if (kbg >= S && !ptx::mbar_wait(&f32_empty[s], ((kbg / S) & 1) ^ 1, p.err, 21)) {
                        go = false;
                        break;
                    }
                    uint8_t *a = st32 + s * C::STAGE32;
                    ptx::mbar_arrive_expect_tx(&f32_full[s], C::STAGE32);
                    if (p.a_kmajor) ptx::tma_load_2d(a, &tmA, &f32_full[s], kb * BK, m0);
                    else ptx::tma_load_2d(a, &tmA, &f32_full[s], m0, kb * BK);
                    if (p.b_kmajor) ptx::tma_load_2d(a + C::A32, &tmB, &f32_full[s], kb * BK, n0);
                    else ptx::tma_load_2d(a + C::A32, &tmB, &f32_full[s], n0, kb * BK);
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
                if (it >= 2 && !ptx::mbar_wait(&acc_empty[b], ((it >> 1) & 1) ^ 1, p.err, 22)) break;
                ptx::tc_fence_after();
                const uint32_t acc = tmem + (uint32_t)(b * BN);
                for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
                    const int s = kbg % S;
                    if (!ptx::mbar_wait(&bf_full[s], (kbg / S) & 1, p.err, 23)) { go = false; break; }
                    ptx::tc_fence_after();
                    const uint32_t st = ptx::smem_u32(stbf + s * C::STAGEBF);
                    const uint64_t ah = ptx::sdesc_kmajor_sw64(st);
                    const uint64_t al = ptx::sdesc_kmajor_sw64(st + C::ABF);
                    const uint64_t bh = ptx::sdesc_kmajor_sw64(st + 2 * C::ABF);
                    const uint64_t bl = ptx::sdesc_kmajor_sw64(st + 2 * C::ABF + C::BBF);
#pragma unroll
                    for (int k = 0; k < BK / 16; k++) {
                        const uint64_t dk = (uint64_t)((k * 32) >> 4);
                        ptx::umma_f16(acc, al + dk, bh + dk, idesc, (kb | k) != 0);
                        ptx::umma_f16(acc, ah + dk, bl + dk, idesc, 1);
                        ptx::umma_f16(acc, ah + dk, bh + dk, idesc, 1);
                    }
                    ptx::umma_commit(&bf_empty[s]);
                }
                if (go) ptx::umma_commit(&acc_full[b]);
            }
        }
    } else if (warp < 6) {   // epilogue: TMEM lane quarter q = warp % 4
        const int q = warp % 4;
        float *stage = epi + q * 32 * 33;
        int it = 0;
        for (int t = blockIdx.x; t < num_tiles; t += gridDim.x, it++) {
            const int b = it & 1;
            if (!ptx::mbar_wait(&acc_full[b], (it >> 1) & 1, p.err, 24)) break;
            ptx::tc_fence_after();
            int tm, tn;
            tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
            const int64_t row0 = (int64_t)tm * BM + q * 32;
            const int64_t n0 = (int64_t)tn * BN;
            for (int c = 0; c < BN; c += 32) {
                uint32_t r[32];
                ptx::tmem_ld_32x32b_x32(tmem + (uint32_t)(b * BN) + ((uint32_t)(q * 32) << 16) + (uint32_t)c, r);
                ptx::tmem_ld_wait();
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
                        for (int rr = 0; rr < 32; rr++) cin[rr] = rr < rows ? p.C[(row0 + rr) * p.ldc + col] : 0.f;
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
    } else {                 // converters: FP32 staging -> hi/lo BF16 tiles
        const int ctid = threadIdx.x - 6 * 32;
        int kbg = 0;
        for (int t = blockIdx.x; t < num_tiles; t += gridDim.x) {
            bool go = true;
            for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
                const int s = kbg % S;
                if (!ptx::mbar_wait(&f32_full[s], (kbg / S) & 1, p.err, 25)) { go = false; break; }
                if (kbg >= S && !ptx::mbar_wait(&bf_empty[s], ((kbg / S) & 1) ^ 1, p.err, 26)) { go = false; break; }
                const uint8_t *a32 = st32 + s * C::STAGE32;
                uint8_t *bf = stbf + s * C::STAGEBF;
                convert_tile<BM>(a32, p.a_kmajor, bf, bf + C::ABF, ctid);
                convert_tile<BN>(a32 + C::A32, p.b_kmajor, bf + 2 * C::ABF, bf + 2 * C::ABF + C::BBF, ctid);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    ptx::mbar_arrive(&f32_empty[s]);
                    ptx::mbar_arrive(&bf_full[s]);
                }
            }
            if (!go) break;
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, C::TMEM_COLS);
    }
}

template <int BN>
gb_status launch(const GemmArgs &g, int *err) {
    using C = Cfg<BN>;
    CUtensorMap tA, tB;
    // op(A) (M x K): K-major when A is row-major (ta = 0); op(B)^T (N x K):
    // K-major when B is stored N x K (tb = 1)
    bool okm;
    if (!g.ta) okm = make_tmap_f32(&tA, g.A, g.K, g.M, g.lda * 4, BK, BM, true);
    else okm = make_tmap_f32(&tA, g.A, g.M, g.K, g.lda * 4, BM, BK, false);
    if (g.tb) okm = okm && make_tmap_f32(&tB, g.B, g.K, g.N, g.ldb * 4, BK, BN, true);
    else okm = okm && make_tmap_f32(&tB, g.B, g.N, g.K, g.ldb * 4, BN, BK, false);
    if (!okm) return set_status(GB_ERR_CUDA, "bf16x3: cuTensorMapEncodeTiled (FP32) failed");
    static std::atomic<uint64_t> attr{0};
    if (device_setup_needed(attr)) {
        GB_CUDA_TRY(cudaFuncSetAttribute(bf16x3_fused_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         C::SMEM));
        device_setup_done(attr);
    }
    Params p;
    p.C = (float *)g.C; p.M = g.M; p.N = g.N; p.ldc = g.ldc;
    p.alpha = (float)g.alpha; p.beta = (float)g.beta; p.semantics = g.semantics;
    p.num_kb = (int)ceil_div(g.K, BK);
    p.tiles_m = (int)ceil_div(g.M, BM);
    p.tiles_n = (int)ceil_div(g.N, BN);
    p.a_kmajor = g.ta ? 0 : 1;
    p.b_kmajor = g.tb ? 1 : 0;
    p.err = err;
    const int tiles = p.tiles_m * p.tiles_n;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    bf16x3_fused_kernel<BN><<<grid, NT, C::SMEM, g.stream>>>(tA, tB, p);
    GB_LAUNCH_CHECK("bf16x3_fused_kernel");
    return ok();
}

}  // namespace fused
}  // namespace

static gb_status two_pass(const GemmArgs &g, int np, int fold_kb);

// Accumulator chunk (k-blocks of 32) from the environment, for measurement.
static int env_chunk(const char *name, int dflt) {
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    const int c = atoi(v);
    return c < 0 ? 0 : c;
}

gb_status launch_sgemm_bf16x3(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    if (g.M > 0x7fffffff / 2 || g.N > 0x7fffffff / 2 || g.K > 0x7fffffff / 2)
        return set_status(GB_ERR_UNSUPPORTED, "bf16x3: dimension too large");
    {
        // fused split: FP32 TMA straight from A and B (16-byte aligned bases,
        // row strides a multiple of 16 bytes)
        // row strides a multiple of 16 bytes).  Used for skinny products
        // (min(M, N) <= 64), where a separate split pass would double the
        // HBM traffic of the streamed operand; large square products keep the
        // two-pass form, whose MMA loop is not slowed by the converters.
        const bool aligned = (g.lda % 4 == 0) && (g.ldb % 4 == 0) && ((uintptr_t)g.A % 16 == 0) &&
                             ((uintptr_t)g.B % 16 == 0);
        const bool skinny = g.M <= 64 || g.N <= 64;
        const char *force = getenv("GB_BF16X3_PATH");   // "fused" / "two-pass": testing and measurement
        const bool use_fused = force ? (force[0] == 'f') : skinny;
        if (aligned && use_fused) {
            int *e = error_word();
            if (!e) return set_status(GB_ERR_OOM, "bf16x3: no device error word");
            if (g.N <= 32) return fused::launch<32>(g, e);
            if (g.N <= 64) return fused::launch<64>(g, e);
            if (g.N <= 128) return fused::launch<128>(g, e);
            return fused::launch<256>(g, e);
        }
    }
    return two_pass(g, 2, env_chunk("GB_BF16X3_FOLD", 0));
}

gb_status launch_sgemm_bf16x6(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    if (g.M > 0x7fffffff / 2 || g.N > 0x7fffffff / 2 || g.K > 0x7fffffff / 2)
        return set_status(GB_ERR_UNSUPPORTED, "bf16x6: dimension too large");
    return two_pass(g, 3, env_chunk("GB_BF16X6_CHUNK", 8));
}

// Stream-K split of the last waves (tiles that do not fill the grid), or
// none: dp_tiles = tiles.  Only when every CTA's share of the split range is
// at least one whole tile, so a split tile has exactly two parts.
// Off unless GB_BF16X3_SK=1: on this GPU the split measured slower than
// whole tiles even where whole tiles waste most of a wave (4096^3, 512
// tiles on 152 SMs: 0.344 vs 0.306 ms per call; 1152 x 4352 x 4096, 153
// tiles: 0.187 vs 0.163 ms), the two parts of a tile fetching its operand
// panels separately (L2 traffic +32 %, DRAM reads +60 %).
static int stream_k_dp_tiles(int tiles, int grid, bool fold) {
    const char *e = getenv("GB_BF16X3_SK");
    if (fold || !(e && e[0] == '1') || grid <= 1) return tiles;
    const int full = tiles / grid, rem = tiles % grid;
    if (rem == 0 || full < 1) return tiles;
    return (full - 1) * grid;
}

template <int NP, int BN, bool FOLD>
static gb_status two_pass_launch(const GemmArgs &g, const PieceMaps &maps, int64_t kp, int *err, int fold_kb,
                                 float *sk_part, int *sk_cnt) {
    using CF = TwoPass<NP, BN>;
    static std::atomic<uint64_t> attr{0};
    if (device_setup_needed(attr)) {
        GB_CUDA_TRY(cudaFuncSetAttribute(bf16x3_gemm_kernel<NP, BN, FOLD>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM_BYTES));
        device_setup_done(attr);
    }
    const int tiles_m = (int)ceil_div(g.M, BM), tiles_n = (int)ceil_div(g.N, BN);
    const int tiles = tiles_m * tiles_n;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    const int dp = sk_part ? stream_k_dp_tiles(tiles, grid, FOLD) : tiles;
    if (dp < tiles) GB_CUDA_TRY(cudaMemsetAsync(sk_cnt, 0, (size_t)grid * sizeof(int), g.stream));
    // half-tile tail when the last wave is at most half full (whole tiles
    // would leave most of the GPU idle for a tile time); GB_BF16X3_HALF=0 off
    int half_start = tiles;
    {
        const char *e = getenv("GB_BF16X3_HALF");
        const int rem = tiles % grid;
        if (!FOLD && BN == 256 && dp == tiles && !(e && e[0] == '0') && rem > 0 && 2 * rem <= grid)
            half_start = tiles - rem;
    }
    EpiParams p{(float *)g.C, g.M, g.N, g.ldc, (float)g.alpha, (float)g.beta, g.semantics, (int)(kp / BK),
                tiles_m, tiles_n, err, FOLD ? fold_kb : 1, dp, sk_part, sk_cnt, half_start};
    bf16x3_gemm_kernel<NP, BN, FOLD><<<grid, NT, CF::SMEM_BYTES, g.stream>>>(maps, p);
    GB_LAUNCH_CHECK("bf16x3_gemm_kernel");
    return ok();
}

// Split pass (NP BF16 pieces per operand, K-major) + MMA kernel; fold_kb > 0
// selects the folding form with that accumulator chunk (in k-blocks of 32).
static gb_status two_pass(const GemmArgs &g, int np, int fold_kb) {
    const int64_t kp = ceil_div(g.K, 64) * 64;   // multiple of BK, zero-padded
    const size_t a_bytes = (size_t)g.M * kp * 2, b_bytes = (size_t)g.N * kp * 2;
    // pieces, then the stream-K part slots (2 per CTA of 128 x 256 FP32) and counters
    const size_t pieces = (np * (a_bytes + b_bytes) + 255) / 256 * 256;
    const bool sk = np == 2 && fold_kb == 0;
    const size_t sk_bytes = sk ? (size_t)sm_count() * 2 * BM * 256 * 4 + (size_t)sm_count() * 4 : 0;
    // Two halves for the pieces, alternating per call on the stream: the split of a call then
    // writes the half the previous call's GEMM is not reading, and is launched to run beside
    // that GEMM (programmatic stream serialization; the GEMM triggers it at its start).  One
    // half, launched in plain order, when the pieces are large or GB_BF16X3_PDL=0.
    const char *pe = getenv("GB_BF16X3_PDL");
    const bool pdl = !(pe && pe[0] == '0') && pieces <= (size_t(8) << 30);
    const int halves = pdl ? 2 : 1;
    unsigned seq = 0;
    size_t ws_size = 0;
    // [half 0 | half 1 | stream-K slots]: the halves at fixed places in the buffer, whatever the
    // size of this call and the last (the buffer only grows after its stream has drained)
    const size_t tail = (sk_bytes + 4096 + 255) / 256 * 256;
    uint8_t *ws = (uint8_t *)workspace(halves * pieces + tail + 512, g.stream, &seq, &ws_size);
    if (!ws) return (gb_status)gb_get_last_status();
    const size_t half = (ws_size - tail) / 2 / 256 * 256;   // >= pieces
    float *sk_part = sk ? (float *)(ws + ws_size - tail) : nullptr;
    int *sk_cnt = sk ? (int *)(ws + ws_size - tail + (size_t)sm_count() * 2 * BM * 256 * 4) : nullptr;
    uint8_t *pw = ws + (pdl ? (size_t)(seq & 1) * half : 0);
    __nv_bfloat16 *ap[3], *bp[3];
    for (int i = 0; i < np; i++) {
        ap[i] = (__nv_bfloat16 *)(pw + i * a_bytes);
        bp[i] = (__nv_bfloat16 *)(pw + np * a_bytes + i * b_bytes);
    }
    cudaLaunchAttribute pdl_attr[1];
    pdl_attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl_attr[0].val.programmaticStreamSerializationAllowed = 1;
    static std::atomic<uint64_t> carve{0};
    if (pdl && device_setup_needed(carve)) {   // the GEMM's shared-memory configuration, so both fit on an SM
        GB_CUDA_TRY(cudaFuncSetAttribute(split_vec_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        GB_CUDA_TRY(cudaFuncSetAttribute(split_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        device_setup_done(carve);
    }
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "bf16x3: no device error word");

    // split: op(A)(m, k) = ta ? A[k*lda + m] : A[m*lda + k]
    //        op(B)^T(n, k) = op(B)(k, n) = tb ? B[n*ldb + k] : B[k*ldb + n]
    const bool vec = g.lda % 4 == 0 && g.ldb % 4 == 0 && (uintptr_t)g.A % 16 == 0 && (uintptr_t)g.B % 16 == 0;
    if (vec) {
        SplitArgs sa;
        memset(&sa, 0, sizeof(sa));
        sa.K = g.K; sa.kp = kp; sa.np = np;
        sa.op[0] = SplitOp{(const float *)g.A, g.lda, g.M, kp / 64, ceil_div(g.M, 64) * (kp / 64), g.ta ? 1 : 0,
                           {ap[0], ap[1], np == 3 ? ap[2] : nullptr}};
        sa.op[1] = SplitOp{(const float *)g.B, g.ldb, g.N, kp / 64, ceil_div(g.N, 64) * (kp / 64), g.tb ? 0 : 1,
                           {bp[0], bp[1], np == 3 ? bp[2] : nullptr}};
        const int64_t blocks = sa.op[0].tiles + sa.op[1].tiles;
        if (blocks > 0x7fffffff) return set_status(GB_ERR_UNSUPPORTED, "bf16x3: operands too large");
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)blocks);
        cfg.blockDim = dim3(256);
        cfg.stream = g.stream;
        cfg.attrs = pdl_attr;
        cfg.numAttrs = pdl ? 1 : 0;
        GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, split_vec_kernel, sa));
        GB_LAUNCH_CHECK("bf16x3 split");
    } else {
        dim3 sgA((unsigned)ceil_div(kp, 32), (unsigned)ceil_div(g.M, 32));
        dim3 sgB((unsigned)ceil_div(kp, 32), (unsigned)ceil_div(g.N, 32));
        if (sgA.y > 65535u || sgB.y > 65535u) return set_status(GB_ERR_UNSUPPORTED, "bf16x3: M or N too large");
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = sgA;
        cfg.blockDim = dim3(256);
        cfg.stream = g.stream;
        cfg.attrs = pdl_attr;
        cfg.numAttrs = pdl ? 1 : 0;
        GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, split_kernel, (const float *)g.A, g.lda, g.ta ? 1 : 0, g.M, g.K, kp,
                                       ap[0], ap[1], np == 3 ? ap[2] : (__nv_bfloat16 *)nullptr));
        GB_LAUNCH_CHECK("bf16x3 split A");
        split_kernel<<<sgB, 256, 0, g.stream>>>((const float *)g.B, g.ldb, g.tb ? 0 : 1, g.N, g.K, kp, bp[0], bp[1],
                                                np == 3 ? bp[2] : nullptr);
        GB_LAUNCH_CHECK("bf16x3 split B");
    }

    const int bn = (np == 3 || fold_kb > 0) ? 128 : 256;
    PieceMaps maps;
    memset(&maps, 0, sizeof(maps));
    bool okm = true;
    for (int i = 0; i < np; i++) {
        okm = okm && make_tmap_bf16(&maps.a[i], ap[i], kp, g.M, kp * 2, BK, BM, 64);
        okm = okm && make_tmap_bf16(&maps.b[i], bp[i], kp, g.N, kp * 2, BK, bn, 64);
        okm = okm && make_tmap_bf16(&maps.bh[i], bp[i], kp, g.N, kp * 2, BK, bn / 2, 64);
    }
    if (!okm) return set_status(GB_ERR_CUDA, "bf16x3: cuTensorMapEncodeTiled failed");
    if (np == 3)
        return fold_kb > 0 ? two_pass_launch<3, 128, true>(g, maps, kp, err, fold_kb, nullptr, nullptr)
                           : two_pass_launch<3, 128, false>(g, maps, kp, err, 0, nullptr, nullptr);
    return fold_kb > 0 ? two_pass_launch<2, 128, true>(g, maps, kp, err, fold_kb, nullptr, nullptr)
                       : two_pass_launch<2, 256, false>(g, maps, kp, err, 0, sk_part, sk_cnt);
}

}  // namespace gb
