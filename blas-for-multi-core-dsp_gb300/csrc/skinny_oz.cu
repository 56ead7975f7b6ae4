// skinny_oz.cu -- FP64 skinny GEMM (irr_thinB / irr_shortA, n <= 64) on the
// tensor cores from integer digits computed in flight.
//
// GB300's FP64 pipe (1.25 TFLOP/s) caps a native FP64 skinny product at
// 2n flops per 8 streamed bytes: ~0.6 TB/s at n = 8, ~0.15 TB/s at n = 32.
// Here X (rows x K, the large operand) is streamed once by TMA and never
// written back; each value is cut, relative to its row's exponent, into
// S = 8 base-64 digits (48 bits; Ozaki, Ogita, Oishi & Rump 2012, integer
// form as in Ootomo, Ozaki & Yokota 2024) that BF16 holds exactly, and the
// digit products run on tcgen05.mma (kind::f16, FP32 accumulate):
//     x_rk = 2^e_r sum_t d_t 2^-6t,   w_kj = 2^f_j sum_u v_u 2^-6u,
//     C_rj ~= 2^(e_r+f_j) sum_{L=2..9} 2^-6L S_L,  S_L = sum_{t+u=L} sum_k d_t v_u.
// Every S_L over a K chunk of 512 is an integer below 8*512*63^2 < 2^24, so
// the FP32 tensor-memory accumulators hold it exactly; at each chunk's end
// the drain warps add the eight level sums into FP64 registers.
//   pass 1: row exponents of X (one read of X), column exponents and the
//           digit slices of W (small);
//   pass 2 (thin_oz_kernel, per 16 columns of W):
//     warp 0     TMA: 128 rows x 32 k of X (FP64) + the 8 digit tiles of W;
//     warps 2-9  converters, two per TMEM lane quarter (one per 16-k box),
//                thread = row: the row's values -> 8 digit slices written
//                into tensor memory (the A operand of the MMA, never in
//                shared memory);
//     warp 1     MMA: the 36 digit pairs t + u <= 9 into 8 level accumulators
//                of 16 columns (two sets, alternating per chunk);
//     warps 10-13 drain: level sums -> FP64, and the epilogue.
// Truncation: digits beyond 2^-48 of the row (or column) maximum and pairs
// below 2^-54 are dropped -- well inside the 2*K*u64 normwise bound.
#include <cuda.h>
#include <cuda_bf16.h>

#include "gb_common.cuh"
#include "sm100_ptx.cuh"

namespace gb {

bool make_tmap_f64(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                   uint32_t box_inner, uint32_t box_outer, bool sw128);
bool make_tmap_bf16(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                    uint32_t box_inner, uint32_t box_outer, int swizzle_bytes);
gb_status ozaki_line_exponents(const double *X, int64_t ld, bool strided, int64_t lines, int64_t len, int *e,
                               cudaStream_t st);

namespace {
namespace thin_oz {

// warps: 0 TMA, 1 MMA, 2-9 converters (two per TMEM lane quarter, one per
// 16-k box), 10-13 drain / epilogue
constexpr int BM = 128, KB = 32, S = 8, NB = 16, STAGES = 4, CHUNK_KB = 16, NCONV = 8, NT = 448;
constexpr uint32_t LV_COLS = S * NB;        // 128: one set of level accumulators (level L at (L-2)*NB)
constexpr uint32_t SLOT0 = 2 * LV_COLS;     // 256: digit slots (digit t at +16(t-1)), two of them
constexpr uint32_t SLOT_COLS = S * 16;      // 128
constexpr uint32_t TMEM_COLS = 512;
constexpr int XS = BM * KB * 8;             // 32 KB: two 16-k boxes of FP64
constexpr int WS = S * NB * KB * 2;         // 8 KB: the 8 digit tiles of W (16 rows of 64 bytes each)
constexpr int STAGE = XS + WS;
constexpr int SMEM = STAGES * STAGE + 1024 /*align*/ + 512 /*barriers*/;

struct OzThinParams {
    int64_t rows, K;
    int n, splits, kchunk_kb, rtiles;       // kchunk_kb: a multiple of CHUNK_KB
    double *C; int64_t cs_r, cs_c;
    double alpha, beta;
    int semantics;
    double *part;                           // splits x rows x NB raw sums (split-K)
    const int *erow, *fcol;
    int *err;
};

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t *>(&v); }

// |x| * 2^(48 - e) as an integer below 2^48 (truncated), and the sign bit.
__device__ __forceinline__ uint64_t scaled_mantissa(double x, int e, uint32_t &sgn) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    sgn = (uint32_t)(b >> 63);
    const int E = (int)((b >> 52) & 0x7FF);
    uint64_t m = b & 0xFFFFFFFFFFFFFull;
    int ex;
    if (E == 0) {
        ex = -1074;
    } else {
        m |= 1ull << 52;
        ex = E - 1075;
    }
    const int shift = ex + 48 - e;   // F = m * 2^shift < 2^48
    if (m == 0 || shift <= -64) return 0;
    return shift >= 0 ? (m << shift) : (m >> (-shift));
}

// digit t (1..8) of F: bits 48-6t .. 53-6t
__device__ __forceinline__ uint32_t digit_of(uint64_t F, int t) { return (uint32_t)(F >> (48 - 6 * t)) & 63u; }

// small non-negative integer -> float, exactly (d < 2^23)
__device__ __forceinline__ float small_int_to_float(uint32_t d) {
    return __int_as_float(0x4B000000 | d) - 8388608.0f;
}

// The 8 digits of F (< 2^48) as floats, most significant first.  The integer
// pipe (half the FP32 lanes of an SM) only cuts F into four 12-bit pieces;
// each piece becomes a float and splits into its two digits with exact FP32
// arithmetic: hi = floor(p / 64) by a round-toward-zero add of 2^23, lo =
// p - 64 hi.
__device__ __forceinline__ void digits_f32(uint64_t F, float (&d)[8]) {
    const uint32_t hi = (uint32_t)(F >> 32), lo = (uint32_t)F;
    const uint32_t p[4] = {hi >> 4, __funnelshift_r(lo, hi, 24) & 0xFFFu, (lo >> 12) & 0xFFFu, lo & 0xFFFu};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float f = small_int_to_float(p[i]);
        const float h = __fadd_rz(f * 0.015625f, 8388608.0f) - 8388608.0f;   // floor(f / 64)
        d[2 * i] = h;
        d[2 * i + 1] = __fmaf_rn(-64.0f, h, f);                               // f - 64 h, exact
    }
}

template <bool XCOLS>
__global__ void __launch_bounds__(NT, 1)
    thin_oz_kernel(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmw, OzThinParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE);
    uint64_t *empty = full + STAGES;
    uint64_t *aready = empty + STAGES;     // [2] digit slots
    uint64_t *aempty = aready + 2;
    uint64_t *lfull = aempty + 2;          // [2] level sets
    uint64_t *lempty = lfull + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(lempty + 2);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int nkb = (int)((p.K + KB - 1) / KB);
    const int units = p.rtiles * p.splits;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1 + NCONV);   // the MMA commit + the converter warps
        }
        for (int a = 0; a < 2; a++) {
            ptx::mbar_init(&aready[a], NCONV);
            ptx::mbar_init(&aempty[a], 1);
            ptx::mbar_init(&lfull[a], 1);
            ptx::mbar_init(&lempty[a], 4);
        }
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&tmx);
        ptx::tma_prefetch_desc(&tmw);
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
                    if (g >= STAGES && !ptx::mbar_wait(&empty[s], ((g / STAGES) & 1) ^ 1, p.err, 61)) {
                        go = false;
                        break;
                    }
                    uint8_t *st = smem + s * STAGE;
                    ptx::mbar_arrive_expect_tx(&full[s], XS + WS);
#pragma unroll
                    for (int b = 0; b < 2; b++) {
                        if (XCOLS) ptx::tma_load_2d(st + b * (XS / 2), &tmx, &full[s], rt * BM, kb * KB + 16 * b);
                        else ptx::tma_load_2d(st + b * (XS / 2), &tmx, &full[s], kb * KB + 16 * b, rt * BM);
                    }
                    ptx::tma_load_2d(st + XS, &tmw, &full[s], kb * KB, 0);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, NB);
            int g = 0, ch = 0;
            bool go = true;
            for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
                const int sp = u % p.splits;
                const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
                for (int c0 = kb0; c0 < kb1 && go; c0 += CHUNK_KB, ch++) {
                    const int lb = ch & 1;
                    if (ch >= 2 && !ptx::mbar_wait(&lempty[lb], ((ch >> 1) & 1) ^ 1, p.err, 62)) {
                        go = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const uint32_t lv = tmem + (uint32_t)(lb * LV_COLS);
                    const int c1 = min(kb1, c0 + CHUNK_KB);
                    for (int kb = c0; kb < c1; kb++, g++) {
                        const int s = g % STAGES, a = g & 1;
                        if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 63) ||
                            !ptx::mbar_wait(&aready[a], (g >> 1) & 1, p.err, 64)) {
                            go = false;
                            break;
                        }
                        ptx::tc_fence_after();
                        const uint32_t wst = ptx::smem_u32(smem + s * STAGE + XS);
                        const uint32_t slot = tmem + SLOT0 + (uint32_t)(a * SLOT_COLS);
#pragma unroll
                        for (int kk = 0; kk < KB / 16; kk++) {
#pragma unroll
                            for (int t = 1; t <= S; t++) {
#pragma unroll
                                for (int v = 1; v + t <= S + 1; v++) {
                                    // digit v of W: rows (v-1)*16 .. of the stage's W tile (1 KB each)
                                    const uint64_t bdesc =
                                        ptx::sdesc_kmajor_sw64(wst + (uint32_t)((v - 1) * NB * 64)) +
                                        (uint64_t)((kk * 32) >> 4);
                                    ptx::umma_f16_ta(lv + (uint32_t)((t + v - 2) * NB),
                                                     slot + (uint32_t)((t - 1) * 16 + kk * 8), bdesc, idesc,
                                                     (kb != c0 || kk != 0 || t != 1) ? 1u : 0u);
                                }
                            }
                        }
                        ptx::umma_commit(&empty[s]);
                        ptx::umma_commit(&aempty[a]);
                    }
                    if (go) ptx::umma_commit(&lfull[lb]);
                }
            }
        }
    } else if (warp < 2 + NCONV) {   // converters: thread = row q*32 + lane, one 16-k box each
        const int q = warp % 4, r = q * 32 + lane, b = (warp - 2) / 4;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int g = 0;
        bool go = true;
        for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
            const int rt = u / p.splits, sp = u - rt * p.splits;
            const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
            const int64_t row = (int64_t)rt * BM + r;
            const int e = row < p.rows ? __ldg(p.erow + row) : 0;
            for (int kb = kb0; kb < kb1; kb++, g++) {
                const int s = g % STAGES, a = g & 1;
                if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 65) ||
                    (g >= 2 && !ptx::mbar_wait(&aempty[a], ((g >> 1) & 1) ^ 1, p.err, 66))) {
                    go = false;
                    break;
                }
                ptx::tc_fence_after();
                const uint8_t *box = smem + s * STAGE + b * (XS / 2);
                const uint32_t slot = tmem + lane_off + SLOT0 + (uint32_t)(a * SLOT_COLS);
                double x[16];
                if (XCOLS) {   // [16 k][128 rows]
                    const double *xs = reinterpret_cast<const double *>(box);
#pragma unroll
                    for (int k = 0; k < 16; k++) x[k] = xs[k * BM + r];
                } else {       // 128 rows of 128 bytes, 16-byte chunks swizzled by row % 8
                    const uint8_t *rowp = box + r * 128;
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        const double2 v = *reinterpret_cast<const double2 *>(rowp + ((c ^ (r & 7)) << 4));
                        x[2 * c] = v.x;
                        x[2 * c + 1] = v.y;
                    }
                }
                uint32_t w[S][8];   // digit t, k pair i -> bf16x2
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    uint32_t s0, s1;
                    float d0[8], d1[8];
                    digits_f32(scaled_mantissa(x[2 * i], e, s0), d0);
                    digits_f32(scaled_mantissa(x[2 * i + 1], e, s1), d1);
                    const uint32_t sm = (s0 << 15) | (s1 << 31);
#pragma unroll
                    for (int t = 0; t < S; t++) w[t][i] = bf16x2_bits(__floats2bfloat162_rn(d0[t], d1[t])) ^ sm;
                }
#pragma unroll
                for (int t = 0; t < S; t++) {
                    uint32_t regs[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) regs[i] = w[t][i];
                    ptx::tmem_st_32x32b_x8(slot + (uint32_t)(t * 16 + b * 8), regs);
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
    } else {                 // drain + epilogue: thread = row q*32 + lane of the tile
        const int q = warp % 4;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int ch = 0;
        bool go = true;
        for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
            const int rt = u / p.splits, sp = u - rt * p.splits;
            const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
            double acc[NB];
#pragma unroll
            for (int j = 0; j < NB; j++) acc[j] = 0.0;
            for (int c0 = kb0; c0 < kb1; c0 += CHUNK_KB, ch++) {
                const int lb = ch & 1;
                if (!ptx::mbar_wait(&lfull[lb], (ch >> 1) & 1, p.err, 67)) { go = false; break; }
                ptx::tc_fence_after();
                // least significant level first, each level sum exact, scaled exactly
#pragma unroll
                for (int L = S + 1; L >= 2; L--) {
                    uint32_t v[16];
                    ptx::tmem_ld_32x32b_x16(tmem + lane_off + (uint32_t)(lb * LV_COLS + (L - 2) * NB), v);
                    ptx::tmem_ld_wait();
                    const double sc = __longlong_as_double((long long)(1023 - 6 * L) << 52);   // 2^-6L
#pragma unroll
                    for (int j = 0; j < NB; j++) acc[j] = fma((double)__uint_as_float(v[j]), sc, acc[j]);
                }
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&lempty[lb]);
            }
            if (!go) break;
            const int64_t row = (int64_t)rt * BM + q * 32 + lane;
            if (row >= p.rows) continue;
            if (p.splits > 1) {
                double *pp = p.part + ((int64_t)sp * p.rows + row) * NB;
#pragma unroll
                for (int j = 0; j < NB; j++) pp[j] = acc[j];
                continue;
            }
            const int er = __ldg(p.erow + row);
            double *cr = p.C + row * p.cs_r;
#pragma unroll
            for (int j = 0; j < NB; j++) {
                if (j >= p.n) break;
                double *cp = cr + (int64_t)j * p.cs_c;
                double v = p.alpha * scalbn(scalbn(acc[j], er), __ldg(p.fcol + j));
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
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// Split-K: sum the parts in order, then scale and apply the epilogue.
__global__ void thin_oz_reduce_kernel(OzThinParams p) {
    const int64_t total = p.rows * p.n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / p.n;
        const int j = (int)(e - r * p.n);
        double s = 0.0;
        for (int sp = 0; sp < p.splits; sp++) s += p.part[((int64_t)sp * p.rows + r) * NB + j];
        double *cp = p.C + r * p.cs_r + (int64_t)j * p.cs_c;
        double v = p.alpha * scalbn(scalbn(s, p.erow[r]), p.fcol[j]);
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

// Digits of W columns j0 .. j0+15 (logical K x n; tw: stored n x K), relative
// to the column exponents: out[(u-1)*16 + jj][k] for u = 1..8, K-major, kp
// columns, zero beyond n and K.
__global__ void wdigits_kernel(const double *__restrict__ W, int64_t ldw, int tw, int n, int j0, int64_t K,
                               int64_t kp, const int *__restrict__ fcol, unsigned short *__restrict__ out) {
    const int64_t total = (int64_t)NB * kp;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int jj = (int)(e / kp);
        const int64_t k = e - (int64_t)jj * kp;
        const int j = j0 + jj;
        double x = 0.0;
        int f = 0;
        if (j < n && k < K) {
            x = tw ? W[(int64_t)j * ldw + k] : W[k * ldw + j];
            f = fcol[jj];
        }
        uint32_t sg;
        const uint64_t F = scaled_mantissa(x, f, sg);
#pragma unroll
        for (int u = 1; u <= S; u++) {
            const uint32_t d = digit_of(F, u);
            const unsigned short h =
                d ? (unsigned short)(__bfloat16_as_ushort(__float2bfloat16_rn(small_int_to_float(d))) | (sg << 15))
                  : 0;
            out[((int64_t)(u - 1) * NB + jj) * kp + k] = h;
        }
    }
}

}  // namespace thin_oz
}  // namespace

// FP64 skinny product through digits on the tensor cores.  X rows x K
// (tx: stored K x rows), W K x n (tw: stored n x K), n <= 64 in passes of 16
// columns, C(r, j) at C[r*cs_r + j*cs_c].  Scratch: `ws` of
// thin_oz_workspace_bytes() bytes.
size_t thin_oz_workspace_bytes(int64_t rows, int64_t K, int n, int splits) {
    const int64_t kp = ceil_div(K, thin_oz::KB) * thin_oz::KB;
    size_t b = (size_t)(rows + 64) * 4 + 256;                            // row exponents (+ column exponents)
    b += (size_t)thin_oz::S * thin_oz::NB * kp * 2 + 256;              // W digit slices of one pass
    if (splits > 1) b += (size_t)splits * rows * thin_oz::NB * 8;      // split-K parts
    (void)n;
    return b;
}

bool thin_oz_eligible(int tx, int64_t ldx, const void *X, int64_t rows, int64_t K) {
    const char *e = getenv("GB_SKINNY_OZ");   // "0": native FP64 kernels (measurement)
    if (e && e[0] == '0') return false;
    (void)tx;
    return K >= 64 && rows < (int64_t(1) << 31) && K < (int64_t(1) << 30) && ldx % 2 == 0 &&
           (uintptr_t)X % 16 == 0;
}

gb_status launch_thin_oz(int64_t rows, int64_t K, const double *X, int64_t ldx, int tx, const double *W, int64_t ldw,
                         int tw, int n, double *C, int64_t cs_r, int64_t cs_c, double alpha, double beta,
                         int semantics, int splits, int64_t kchunk, void *ws, cudaStream_t st) {
    using namespace thin_oz;
    const int64_t kp = ceil_div(K, KB) * KB;
    uint8_t *w8 = (uint8_t *)ws;
    int *erow = (int *)w8;
    int *fcol = erow + rows;   // up to 64 columns
    size_t off = ((size_t)(rows + 64) * 4 + 255) / 256 * 256;
    unsigned short *wd = (unsigned short *)(w8 + off);
    off += ((size_t)S * NB * kp * 2 + 255) / 256 * 256;
    double *part = splits > 1 ? (double *)(w8 + off) : nullptr;
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "skinny: no device error word");

    gb_status s = ozaki_line_exponents(X, ldx, tx != 0, rows, K, erow, st);
    if (s != GB_OK) return s;
    s = ozaki_line_exponents(W, ldw, tw == 0, n, K, fcol, st);
    if (s != GB_OK) return s;

    CUtensorMap tx_map, tw_map;
    const bool okx = tx ? make_tmap_f64(&tx_map, X, (uint64_t)rows, (uint64_t)K, (uint64_t)ldx * 8, BM, 16, false)
                        : make_tmap_f64(&tx_map, X, (uint64_t)K, (uint64_t)rows, (uint64_t)ldx * 8, 16, BM, true);
    const bool okw = make_tmap_bf16(&tw_map, wd, (uint64_t)kp, (uint64_t)S * NB, (uint64_t)kp * 2, KB, S * NB, 64);
    if (!okx || !okw) return set_status(GB_ERR_CUDA, "skinny: cuTensorMapEncodeTiled failed");

    static bool attr = false;
    if (!attr) {
        GB_CUDA_TRY(cudaFuncSetAttribute(thin_oz_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
        GB_CUDA_TRY(cudaFuncSetAttribute(thin_oz_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
        attr = true;
    }
    const int rtiles = (int)ceil_div(rows, BM);
    const int units = rtiles * splits;
    const int grid = units < sm_count() ? units : sm_count();
    for (int j0 = 0; j0 < n; j0 += NB) {   // 16 columns of W per pass over X
        const int nc = n - j0 < NB ? n - j0 : NB;
        const int blocks = (int)(ceil_div((int64_t)NB * kp, 256) < 2 * sm_count() ? ceil_div((int64_t)NB * kp, 256)
                                                                                    : 2 * sm_count());
        wdigits_kernel<<<blocks, 256, 0, st>>>(W, ldw, tw, n, j0, K, kp, fcol + j0, wd);
        GB_LAUNCH_CHECK("wdigits_kernel");
        OzThinParams p{rows, K, nc, splits, (int)(kchunk / KB), rtiles,
                       C + j0 * cs_c, cs_r, cs_c, alpha, beta, semantics, part, erow, fcol + j0, err};
        if (tx) thin_oz_kernel<true><<<grid, NT, SMEM, st>>>(tx_map, tw_map, p);
        else thin_oz_kernel<false><<<grid, NT, SMEM, st>>>(tx_map, tw_map, p);
        GB_LAUNCH_CHECK("thin_oz_kernel");
        if (splits > 1) {
            const int rb = (int)(ceil_div(rows * nc, 256) < 4 * sm_count() ? ceil_div(rows * nc, 256) : 4 * sm_count());
            thin_oz_reduce_kernel<<<rb, 256, 0, st>>>(p);
            GB_LAUNCH_CHECK("thin_oz_reduce_kernel");
        }
    }
    return ok();
}

}  // namespace gb
