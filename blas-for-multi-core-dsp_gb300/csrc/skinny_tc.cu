// skinny_tc.cu -- FP32 skinny GEMM with 8 < n <= 64 as 3xBF16 on tcgen05.
//
// Same problem as skinny.cu (irr_thinB / irr_shortA, the large operand X is
// rows x K, the small one W is K x n, C(r, j) at C[r*cs_r + j*cs_c]), for a
// small dimension where FP32 FFMA could no longer keep up with HBM: at n = 64
// the products need 8x the FFMA rate that streaming X at full bandwidth
// allows.  The products run on the tensor cores as
//     x_hi*w_hi + x_hi*w_lo + x_lo*w_hi      (BF16 pieces, FP32 accumulate)
// and X is split in flight, never written back to HBM:
//   * warp 0 (TMA) streams stages of 128 rows x 64 k of X (two 32-k boxes:
//     row-major X as 128-byte swizzled rows, K-major X as [32 k][128 rows])
//     and the matching 64-k tiles of W_hi / W_lo (W is split once per call by
//     wsplit_kernel into K-major BF16 pieces, a few hundred KB in L2);
//   * warps 2-5 (one per TMEM lane quarter) each own 32 rows: a thread reads
//     its row's 64 values from shared memory, splits them and writes hi / lo
//     straight into tensor memory (tcgen05.st) -- the MMA reads A from TMEM,
//     so the split pieces never touch shared memory;
//   * warp 1 issues tcgen05.mma (M = 128, N = NB, K = 16, A from TMEM, B from
//     shared memory) into one of two TMEM accumulators of NB columns;
//   * warps 6-9 read the finished accumulator (tcgen05.ld) and apply
//     alpha / beta, or write split-K partials for skinny_reduce_kernel.
// Shared-memory traffic per X value is the TMA write and one read (8 bytes).
//
// Row-major X whose leading dimension is not a multiple of 4 floats cannot be
// described by one tensor map (row starts fall on different 16-byte phases),
// so its rows are taken in four classes r = 4i + c: class c has a 16-byte
// aligned base X + c*ldx - d_c (d_c = c*ldx mod 4) and a row stride of
// 4*ldx floats, and its coordinate x holds k = x - d_c.  The W pieces are
// stored once per phase d, shifted so the same aligned tile coordinate yields
// W(k) for that class; values at k < 0 (the tail of the previous row) are
// zeroed by the converters.
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

constexpr int BM = 128, KS = 64, STAGES = 4, ASLOTS = 4, NT = 320;
constexpr int WOFF = 64;              // W pieces: element k of phase d at column k + WOFF + d
constexpr uint32_t A_COL0 = 128;      // A slot i at TMEM columns 128 + 64 i (hi: +0..31, lo: +32..63)
constexpr uint32_t TMEM_COLS = 512;   // accumulators at columns [0, 2 NB)

// K-major X with ldx % 4 != 0: four classes of k-lines (k = 4i + c), each a
// box of 132 x 16 (rows x lines) -- 128 rows plus the class's phase d_c
constexpr int CB_W = BM + 4, CB_L = KS / 4, CB_BYTES = CB_W * CB_L * 4;   // 8448 bytes

template <int NB>
struct Cfg {
    static constexpr int XS = 4 * CB_BYTES;  // 33 KB: room for either X form (two 16 KB boxes or four class boxes)
    static constexpr int WP = NB * KS * 2;   // one BF16 piece of W (NB rows of 128 bytes)
    static constexpr int STAGE = (XS + 2 * WP + 1023) / 1024 * 1024;
    static constexpr int SMEM = STAGES * STAGE + 1024 /*align*/ + 512 /*barriers*/;
};

struct TcParams {
    int64_t rows, K;
    int n, splits, kchunk_st;             // stages of 64 k per split
    int nst;                              // stages covering K (+ the largest phase)
    int rstride;                          // 4 with row classes, else 1
    int64_t cls_rows[4];                  // rows in class c
    int cls_delta[4];
    int cls_u0[5];                        // first unit of class c
    int kdelta[4];                        // K-major X in k-line classes: phase of class c
    float *C; int64_t cs_r, cs_c;
    float alpha, beta;
    int semantics;
    float *part;
    int *err;
};

struct Maps {
    CUtensorMap x[4], wh[4], wl[4];
};

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) {
    return *reinterpret_cast<uint32_t *>(&v);
}

// unit u -> class c, row tile rt (within the class), split sp
__device__ __forceinline__ void unit_coords(const TcParams &p, int u, int &c, int &rt, int &sp) {
    c = 0;
    while (c < 3 && u >= p.cls_u0[c + 1]) c++;
    const int v = u - p.cls_u0[c];
    rt = v / p.splits;
    sp = v - rt * p.splits;
}

// XL: 0 row-major X (rows in classes when ldx % 4 != 0), 1 K-major X with
// ldx % 4 == 0, 2 K-major X in k-line classes
template <int NB, int XL>
__global__ void __launch_bounds__(NT, 1) thin_tc_kernel(const __grid_constant__ Maps maps, TcParams p) {
    constexpr bool XCOLS = XL != 0;
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
    const int units = p.cls_u0[4];

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
                int c, rt, sp;
                unit_coords(p, u, c, rt, sp);
                const int s0 = sp * p.kchunk_st, s1 = min(p.nst, s0 + p.kchunk_st);
                for (int ks = s0; ks < s1; ks++, g++) {
                    const int s = g % STAGES;
                    if (g >= STAGES && !ptx::mbar_wait(&empty[s], ((g / STAGES) & 1) ^ 1, p.err, 51)) {
                        go = false;
                        break;
                    }
                    uint8_t *st = smem + s * C::STAGE;
                    if (XL == 2) {
                        ptx::mbar_arrive_expect_tx(&full[s], 4 * CB_BYTES + 2 * C::WP);
#pragma unroll
                        for (int kc = 0; kc < 4; kc++)
                            ptx::tma_load_2d(st + kc * CB_BYTES, &maps.x[kc], &full[s], rt * BM, ks * CB_L);
                    } else {
                        ptx::mbar_arrive_expect_tx(&full[s], 2 * BM * 32 * 4 + 2 * C::WP);
#pragma unroll
                        for (int b = 0; b < 2; b++) {
                            if (XCOLS) ptx::tma_load_2d(st + b * BM * 128, &maps.x[c], &full[s], rt * BM, ks * KS + 32 * b);
                            else ptx::tma_load_2d(st + b * BM * 128, &maps.x[c], &full[s], ks * KS + 32 * b, rt * BM);
                        }
                    }
                    ptx::tma_load_2d(st + C::XS, &maps.wh[c], &full[s], ks * KS + WOFF, 0);
                    ptx::tma_load_2d(st + C::XS + C::WP, &maps.wl[c], &full[s], ks * KS + WOFF, 0);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, NB);
            int g = 0, it = 0;
            bool go = true;
            for (int u = blockIdx.x; u < units && go; u += gridDim.x, it++) {
                int c, rt, sp;
                unit_coords(p, u, c, rt, sp);
                const int s0 = sp * p.kchunk_st, s1 = min(p.nst, s0 + p.kchunk_st);
                const int b = it & 1;
                if (it >= 2 && !ptx::mbar_wait(&acce[b], ((it >> 1) & 1) ^ 1, p.err, 52)) break;
                ptx::tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(b * NB);
                for (int ks = s0; ks < s1; ks++, g++) {
                    const int s = g % STAGES, a = g % ASLOTS;
                    if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 53) ||
                        !ptx::mbar_wait(&aready[a], (g / ASLOTS) & 1, p.err, 54)) {
                        go = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const uint32_t st = ptx::smem_u32(smem + s * C::STAGE);
                    const uint64_t bh = ptx::sdesc_kmajor_sw128(st + C::XS);
                    const uint64_t bl = ptx::sdesc_kmajor_sw128(st + C::XS + C::WP);
                    const uint32_t ah = tmem + A_COL0 + (uint32_t)(a * 64), al = ah + 32u;
#pragma unroll
                    for (int kk = 0; kk < KS / 16; kk++) {
                        const uint64_t dk = (uint64_t)((kk * 32) >> 4);   // 16 BF16 = 32 bytes along K
                        const uint32_t ck = (uint32_t)(kk * 8);           // 16 BF16 = 8 TMEM columns
                        ptx::umma_f16_ta(d, al + ck, bh + dk, idesc, (ks != s0 || kk != 0) ? 1u : 0u);
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
            int c, rt, sp;
            unit_coords(p, u, c, rt, sp);
            const int s0 = sp * p.kchunk_st, s1 = min(p.nst, s0 + p.kchunk_st);
            const int delta = p.cls_delta[c];
            for (int ks = s0; ks < s1; ks++, g++) {
                const int s = g % STAGES, a = g % ASLOTS;
                if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 55) ||
                    (g >= ASLOTS && !ptx::mbar_wait(&aempty[a], ((g / ASLOTS) & 1) ^ 1, p.err, 56))) {
                    go = false;
                    break;
                }
                ptx::tc_fence_after();
                const uint8_t *st = smem + s * C::STAGE;
#pragma unroll
                for (int b = 0; b < 2; b++) {   // 32 k per box: hi to columns +16b.., lo to +32+16b..
                    float x[32];
                    const uint8_t *box = st + b * BM * 128;
                    if (XL == 2) {   // k = 32b + kk: class kk % 4, line 8b + kk / 4, at row r + d_class
                        const float *xs = reinterpret_cast<const float *>(st);
#pragma unroll
                        for (int kk = 0; kk < 32; kk++) {
                            const int kc = kk & 3;
                            x[kk] = xs[kc * (CB_BYTES / 4) + (8 * b + kk / 4) * CB_W + r + p.kdelta[kc]];
                        }
                    } else if (XCOLS) {
                        const float *xs = reinterpret_cast<const float *>(box);
#pragma unroll
                        for (int k = 0; k < 32; k++) x[k] = xs[k * BM + r];
                    } else {
                        const uint8_t *row = box + r * 128;
#pragma unroll
                        for (int cc = 0; cc < 8; cc++) {
                            const float4 v = *reinterpret_cast<const float4 *>(row + ((cc ^ (r & 7)) << 4));
                            x[4 * cc] = v.x; x[4 * cc + 1] = v.y; x[4 * cc + 2] = v.z; x[4 * cc + 3] = v.w;
                        }
                    }
                    if (ks == 0 && b == 0 && delta > 0) {   // coordinates below d_c are the previous row
#pragma unroll
                        for (int k = 0; k < 3; k++)
                            if (k < delta) x[k] = 0.f;
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
                    // hi words of this box -> slot + 16b .. +15, lo -> slot + 32 + 16b ..
                    uint32_t hw[16], lw[16];
#pragma unroll
                    for (int i = 0; i < 16; i++) { hw[i] = pk[i]; lw[i] = pk[16 + i]; }
                    ptx::tmem_st_32x32b_x16(tmem + lane_off + A_COL0 + (uint32_t)(a * 64 + 16 * b), hw);
                    ptx::tmem_st_32x32b_x16(tmem + lane_off + A_COL0 + (uint32_t)(a * 64 + 32 + 16 * b), lw);
                }
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
            int c, rt, sp;
            unit_coords(p, u, c, rt, sp);
            const int b = it & 1;
            if (!ptx::mbar_wait(&accf[b], (it >> 1) & 1, p.err, 57)) break;
            ptx::tc_fence_after();
            float acc[NB];
#pragma unroll
            for (int cc = 0; cc < NB; cc += 16) {
                uint32_t v[16];
                ptx::tmem_ld_32x32b_x16(tmem + lane_off + (uint32_t)(b * NB + cc), v);
                ptx::tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 16; j++) acc[cc + j] = __uint_as_float(v[j]);
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&acce[b]);
            const int64_t i = (int64_t)rt * BM + q * 32 + lane;   // row within the class
            if (i >= p.cls_rows[c]) continue;
            const int64_t row = i * p.rstride + c;
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

// W (logical K x n; tw: stored n x K) -> hi / lo BF16 pieces [nb][lp] for
// each phase d < nphase: piece_d[j][x] = W(x - WOFF - d, j), zero outside
// 0 <= k < K, j < n.  K-major, 128-byte rows of 64 k.
__global__ void wsplit_kernel(const float *__restrict__ W, int64_t ldw, int tw, int n, int64_t K, int64_t lp, int nb,
                              int nphase, __nv_bfloat16 *__restrict__ pieces) {
    const int64_t per = (int64_t)nb * lp;
    const int64_t total = per * nphase;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = e / per, r = e - d * per;
        const int64_t j = r / lp, x = r - j * lp;
        const int64_t k = x - WOFF - d;
        float v = 0.f;
        if (j < n && k >= 0 && k < K) v = tw ? W[j * ldw + k] : W[k * ldw + j];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        __nv_bfloat16 *hi = pieces + d * 2 * per, *lo = hi + per;
        hi[r] = h;
        lo[r] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

template <int NB, int XL>
gb_status launch_nb(const ThinTcArgs &a, const Maps &maps, const TcParams &tp, int grid) {
    static std::atomic<uint64_t> attr{0};
    if (device_setup_needed(attr)) {
        GB_CUDA_TRY(cudaFuncSetAttribute(thin_tc_kernel<NB, XL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Cfg<NB>::SMEM));
        device_setup_done(attr);
    }
    thin_tc_kernel<NB, XL><<<grid, NT, Cfg<NB>::SMEM, a.stream>>>(maps, tp);
    GB_LAUNCH_CHECK("thin_tc_kernel");
    return ok();
}

}  // namespace thin_tc
}  // namespace

bool thin_tc_row_classes(int tx, int64_t ldx) { return !tx && ldx % 4 != 0; }

// stages of 64 k covering K shifted by the largest phase
int64_t thin_tc_stages(int64_t K, bool classes) { return ceil_div(K + (classes ? 3 : 0), thin_tc::KS); }

static int64_t pieces_len(int64_t K, bool classes) { return thin_tc::WOFF + thin_tc_stages(K, classes) * thin_tc::KS; }

size_t thin_tc_wpieces_bytes(int nb, int64_t K, bool classes) {
    return (size_t)(classes ? 4 : 1) * 2 * nb * pieces_len(K, classes) * 2;
}

gb_status launch_thin_tc(const ThinTcArgs &a) {
    using namespace thin_tc;
    const bool classes = thin_tc_row_classes(a.tx, a.ldx);
    const bool kcls = a.tx && a.ldx % 4 != 0;   // K-major X in k-line classes
    const int nphase = classes ? 4 : 1;
    const int64_t lp = pieces_len(a.K, classes);
    __nv_bfloat16 *pieces = (__nv_bfloat16 *)a.wpieces;
    {
        const int64_t total = (int64_t)nphase * a.nb * lp;
        const int blocks = (int)(ceil_div(total, 256) < 2 * sm_count() ? ceil_div(total, 256) : 2 * sm_count());
        wsplit_kernel<<<blocks, 256, 0, a.stream>>>(a.W, a.ldw, a.tw, a.n, a.K, lp, a.nb, nphase, pieces);
        GB_LAUNCH_CHECK("wsplit_kernel");
    }
    Maps maps;
    memset(&maps, 0, sizeof(maps));
    TcParams tp;
    memset(&tp, 0, sizeof(tp));
    tp.rows = a.rows; tp.K = a.K; tp.n = a.n; tp.splits = a.splits;
    tp.nst = (int)thin_tc_stages(a.K, classes);
    tp.kchunk_st = (int)(a.kchunk / KS);
    tp.rstride = classes ? 4 : 1;
    bool okm = true;
    int u = 0;
    for (int c = 0; c < 4; c++) {
        tp.cls_u0[c] = u;
        int64_t rows_c;
        int delta = 0;
        const float *base = a.X;
        if (!classes) {
            rows_c = c == 0 ? a.rows : 0;
        } else {
            rows_c = a.rows > c ? (a.rows - c + 3) / 4 : 0;
            delta = (int)((c * a.ldx) % 4);
            base = a.X + c * a.ldx - delta;
        }
        tp.cls_rows[c] = rows_c;
        tp.cls_delta[c] = delta;
        u += (int)(ceil_div(rows_c, BM) * a.splits);
        if (rows_c == 0) continue;
        const __nv_bfloat16 *wh = pieces + (int64_t)delta * 2 * a.nb * lp, *wl = wh + (int64_t)a.nb * lp;
        if (a.tx && kcls) {
            for (int kc = 0; kc < 4; kc++) {
                const int64_t lines = a.K > kc ? (a.K - kc + 3) / 4 : 0;
                const int kd = (int)((kc * a.ldx) % 4);
                tp.kdelta[kc] = kd;
                if (lines == 0) {   // a class with no lines: never read beyond K (zero fill), map class 0
                    okm = okm && make_tmap_f32(&maps.x[kc], a.X, (uint64_t)(a.rows + 4), 1, (uint64_t)a.ldx * 16,
                                               CB_W, CB_L, false);
                    continue;
                }
                okm = okm && make_tmap_f32(&maps.x[kc], a.X + kc * a.ldx - kd, (uint64_t)(a.rows + kd),
                                           (uint64_t)lines, (uint64_t)a.ldx * 16, CB_W, CB_L, false);
            }
        } else if (a.tx)
            okm = okm && make_tmap_f32(&maps.x[c], base, (uint64_t)a.rows, (uint64_t)a.K, (uint64_t)a.ldx * 4, BM,
                                       32, false);
        else
            okm = okm && make_tmap_f32(&maps.x[c], base, (uint64_t)(a.K + delta), (uint64_t)rows_c,
                                       (uint64_t)a.ldx * 4 * (classes ? 4 : 1), 32, BM, true);
        okm = okm && make_tmap_bf16(&maps.wh[c], wh, (uint64_t)lp, (uint64_t)a.nb, (uint64_t)lp * 2, KS,
                                    (uint32_t)a.nb, 128);
        okm = okm && make_tmap_bf16(&maps.wl[c], wl, (uint64_t)lp, (uint64_t)a.nb, (uint64_t)lp * 2, KS,
                                    (uint32_t)a.nb, 128);
    }
    tp.cls_u0[4] = u;
    if (!okm) return set_status(GB_ERR_CUDA, "skinny: cuTensorMapEncodeTiled failed");
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "skinny: no device error word");
    tp.C = a.C; tp.cs_r = a.cs_r; tp.cs_c = a.cs_c; tp.alpha = a.alpha; tp.beta = a.beta;
    tp.semantics = a.semantics; tp.part = a.part; tp.err = err;
    const int grid = u < sm_count() ? u : sm_count();
    if (grid == 0) return ok();
    const int xl = !a.tx ? 0 : (kcls ? 2 : 1);
    switch (a.nb * 4 + xl) {
        case 64: return launch_nb<16, 0>(a, maps, tp, grid);
        case 65: return launch_nb<16, 1>(a, maps, tp, grid);
        case 66: return launch_nb<16, 2>(a, maps, tp, grid);
        case 128: return launch_nb<32, 0>(a, maps, tp, grid);
        case 129: return launch_nb<32, 1>(a, maps, tp, grid);
        case 130: return launch_nb<32, 2>(a, maps, tp, grid);
        case 256: return launch_nb<64, 0>(a, maps, tp, grid);
        case 257: return launch_nb<64, 1>(a, maps, tp, grid);
        case 258: return launch_nb<64, 2>(a, maps, tp, grid);
        default: return set_status(GB_ERR_UNSUPPORTED, "skinny: no tensor-core tile for n = %d", a.n);
    }
}

}  // namespace gb
