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
// Row exponents are taken per K chunk of 256 (e_rc: max |x| < 2^e_rc over
// row r's 256 values), so X is read once from HBM: a scan of the chunk
// through a second TMA ring finds them, and the conversion re-reads the same
// chunk from L2 one chunk later.  Every S_L over a chunk is an integer below
// 8*256*63^2 < 2^24, so the FP32 tensor-memory accumulators hold it exactly;
// at each chunk's end the drain warps combine the eight level sums into one
// exact 64-bit integer per output and add it, scaled by 2^(e_rc - 54), into
// FP64 registers (relative to the row's running maximum exponent): one
// FP64 conversion and one FMA per output and chunk, as GB300's FP64 pipe is
// narrow.
//   pass 1: column exponents and the digit slices of W (small);
//   pass 2 (thin_oz_kernel, per 16 or 32 columns of W -- one or two groups):
//     warp 0     TMA: 128 rows x 32 k of X (FP64) + the 8 digit tiles of W
//                (or, for leading dimensions TMA cannot take, all lanes
//                copying X by 8-byte cp.async into the same layout);
//     warp 14    TMA: the same X boxes, one chunk ahead, for the scan;
//     warp 15    scan of chunk c+1 (four rows per lane: the maximum |x| bit
//                pattern -> e_rc in shared memory);
//     warps 10-13 drain chunk c: level sums -> FP64, and the epilogue;
//     warps 2-9  converters, two per TMEM lane quarter (one per 16-k box),
//                thread = row: the row's values -> 8 digit slices written
//                into tensor memory (the A operand of the MMA, never in
//                shared memory);
//     warp 1     MMA: one MMA per digit t of X against W's digits
//                u = 1 .. 9-t of all the pass's columns at once
//                (N = PW(9-t), PW = 16 or 32): W's digit rows lie in shared
//                memory in the order [u = 8 .. 1][column], so the pair (t, u)
//                lands in accumulator column block 9 - t - u for every t,
//                i.e. level L = t + u at columns PW(9-L) .. PW(9-L)+PW-1;
//                one group: two level sets alternate per chunk; two groups:
//                one 256-column set, handed back by the drain between chunks.
// The exponent slots of a chunk are freed separately by the converters and
// by the drain (each arrives in chunk order on its own barrier), so that
// converters two chunks ahead of a drain held up in an epilogue cannot
// release a slot the drain has not read.
// Truncation: digits beyond 2^-48 of the chunk's row maximum (or the column
// maximum) and pairs below 2^-54 are dropped -- well inside the 2*K*u64
// normwise bound.  An output whose row of X or column of W holds an Inf or a
// NaN is recomputed as a plain FP64 dot product, so non-finite values
// propagate.
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

// warps: 0 TMA (converter stages), 1 MMA, 2-9 converters (two per TMEM lane
// quarter, one per 16-k box), 10-13 drain / epilogue, 14 TMA (scan ring),
// 15 scan
constexpr int BM = 128, KB = 32, S = 8, NB = 16, SSTAGES = 2, CHUNK_KB = 8, NCONV = 8, NT = 512;
constexpr uint32_t LV_COLS = S * NB;        // 128: one set of level accumulators (level L at (S+1-L)*NB)
constexpr uint32_t SLOT0 = 2 * LV_COLS;     // 256: digit slots (digit t at +16(t-1)), two of them
constexpr uint32_t SLOT_COLS = S * 16;      // 128
constexpr uint32_t TMEM_COLS = 512;
constexpr int XS = BM * KB * 8;             // 32 KB: two 16-k boxes of FP64
constexpr int BAR_BYTES = 512, EXP_BYTES = 2 * BM * 4;
constexpr int NO_EXP = -100000;             // chunk exponent of an all-zero row chunk

// NG groups of 16 columns of W per pass.  NG = 1: two level sets alternate per
// chunk (tensor memory: 2 x 128 level columns + 2 x 128 digit-slot columns);
// NG = 2: one level set per column group, drained in place between chunks.
template <int NG>
struct Cfg {
    static constexpr int STAGES = NG == 1 ? 4 : 3;
    static constexpr int WS = NG * S * NB * KB * 2;   // 8 KB per group: 8 digit tiles of 16 rows x 64 bytes, u = 8 .. 1
    static constexpr int STAGE = XS + WS;
    static constexpr int SMEM = STAGES * STAGE + SSTAGES * XS + 1024 /*align*/ + BAR_BYTES + EXP_BYTES;
    static_assert(SMEM <= 232448, "shared memory");
};

struct OzThinParams {
    int64_t rows, K;
    int n, splits, kchunk_kb, rtiles;       // kchunk_kb: a multiple of CHUNK_KB; n <= 16 NG
    int pw;                                 // columns of the pass: 16 NG
    double *C; int64_t cs_r, cs_c;
    double alpha, beta;
    int semantics;
    double *part;                           // splits x rows x pw sums (split-K)
    int *nfrow;                             // split-K: rows that hold an Inf / NaN
    const int *fcol;
    int *err;
    // operands, for the outputs that a non-finite row or column reaches
    const double *X, *W;
    int64_t ldx, ldw;
    int tx, tw, j0;
};

// The (unit, chunk) pairs of this CTA in order: unit u = (row tile, split),
// chunks of CHUNK_KB k blocks from the split's first.
struct Walk {
    int u, c0, kb1;
    __device__ __forceinline__ void set(const OzThinParams &p, int nkb) {
        c0 = (u % p.splits) * p.kchunk_kb;
        kb1 = min(nkb, c0 + p.kchunk_kb);
    }
    __device__ __forceinline__ void first(const OzThinParams &p, int nkb) {
        u = blockIdx.x;
        set(p, nkb);
    }
    __device__ __forceinline__ int c1() const { return min(kb1, c0 + CHUNK_KB); }
    __device__ __forceinline__ bool last() const { return c0 + CHUNK_KB >= kb1; }
    __device__ __forceinline__ void next(const OzThinParams &p, int nkb) {
        c0 += CHUNK_KB;
        if (c0 >= kb1) {
            u += gridDim.x;
            set(p, nkb);
        }
    }
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

// 64-bit right shift whose amounts of 64 and more give zero (PTX clamps them).
__device__ __forceinline__ uint64_t shr64(uint64_t v, uint32_t s) {
    uint64_t r;
    asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(v), "r"(s));
    return r;
}

// scaled_mantissa() for rows with e >= -974, from the high and low words of
// x: every finite x of the row has a right shift rs = 1027 + e - E >= 5 (its
// biased exponent E <= e + 1022).  Zeros and subnormals (E = 0) get the
// implicit bit set wrongly, but with rs >= 53 it shifts out with the rest.
__device__ __forceinline__ uint64_t scaled_mantissa_fast(uint32_t hi, uint32_t lo, int e1027) {
    const uint32_t rs = (uint32_t)(e1027 - (int)((hi >> 20) & 0x7FFu));
    return shr64(((uint64_t)((hi & 0xFFFFFu) | 0x100000u) << 32) | lo, rs);
}

// the two halves as a bf16x2 word (exact: the digits are small integers)
__device__ __forceinline__ uint32_t f2_bf16x2(uint64_t v) {
    float lo, hi;
    ptx::f2_unpack(v, lo, hi);
    return bf16x2_bits(__floats2bfloat162_rn(lo, hi));
}

// The 8 digits of two values' F (< 2^48), most significant first, each a float
// carrying the sign of its x (the sign bit of its `hi`), as bf16x2 words w[t]
// (value 0 in the low half).  The integer pipe only cuts F into three pieces
// of 18, 18 and 12 bits and writes each into the low bits of C = +-2^23 (a
// float +-(2^23 + p)); FP32 arithmetic, exact throughout and done for both
// values at once, does the rest: f = +-p, then repeatedly
// hi = trunc(f / 2^s) by a round-toward-zero fma onto +-2^23 and f - 2^s hi.
__device__ __forceinline__ void digit_words(uint64_t F0, uint32_t hi0, uint64_t F1, uint32_t hi1, uint32_t (&w)[S]) {
    const uint32_t C0 = (hi0 & 0x80000000u) | 0x4B000000u, C1 = (hi1 & 0x80000000u) | 0x4B000000u;
    const uint64_t M = ptx::f2_pack(__uint_as_float(C0), __uint_as_float(C1));
    const uint32_t fh0 = (uint32_t)(F0 >> 32), fl0 = (uint32_t)F0, fh1 = (uint32_t)(F1 >> 32), fl1 = (uint32_t)F1;
    const uint64_t f0 = ptx::f2_sub(ptx::f2_pack(__uint_as_float(__funnelshift_r(fl0, fh0, 30) | C0),   // bits 30..47
                                       __uint_as_float(__funnelshift_r(fl1, fh1, 30) | C1)), M);
    const uint64_t f1 = ptx::f2_sub(ptx::f2_pack(__uint_as_float(((fl0 >> 12) & 0x3FFFFu) | C0),        // bits 12..29
                                       __uint_as_float(((fl1 >> 12) & 0x3FFFFu) | C1)), M);
    const uint64_t f2 = ptx::f2_sub(ptx::f2_pack(__uint_as_float((fl0 & 0xFFFu) | C0),                  // bits 0..11
                                       __uint_as_float((fl1 & 0xFFFu) | C1)), M);
    const uint64_t s12 = ptx::f2_pack(1.0f / 4096.0f, 1.0f / 4096.0f), m12 = ptx::f2_pack(-4096.0f, -4096.0f);
    const uint64_t s6 = ptx::f2_pack(0.015625f, 0.015625f), m6 = ptx::f2_pack(-64.0f, -64.0f);
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const uint64_t f = i ? f1 : f0;
        const uint64_t h = ptx::f2_sub(ptx::f2_fma_rz(f, s12, M), M);
        const uint64_t r = ptx::f2_fma_rn(m12, h, f);
        const uint64_t h2 = ptx::f2_sub(ptx::f2_fma_rz(r, s6, M), M);
        w[3 * i] = f2_bf16x2(h);
        w[3 * i + 1] = f2_bf16x2(h2);
        w[3 * i + 2] = f2_bf16x2(ptx::f2_fma_rn(m6, h2, r));
    }
    const uint64_t h = ptx::f2_sub(ptx::f2_fma_rz(f2, s6, M), M);
    w[6] = f2_bf16x2(h);
    w[7] = f2_bf16x2(ptx::f2_fma_rn(m6, h, f2));
}

// The 16 values of one box row -> 8 digit slices of 8 bf16x2 words.
template <bool FAST>
__device__ __forceinline__ void convert16(const double (&x)[16], int e, uint32_t (&w)[S][8]) {
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint64_t b0 = (uint64_t)__double_as_longlong(x[2 * i]), b1 = (uint64_t)__double_as_longlong(x[2 * i + 1]);
        const uint32_t h0 = (uint32_t)(b0 >> 32), h1 = (uint32_t)(b1 >> 32);
        uint64_t F0, F1;
        if (FAST) {
            F0 = scaled_mantissa_fast(h0, (uint32_t)b0, 1027 + e);
            F1 = scaled_mantissa_fast(h1, (uint32_t)b1, 1027 + e);
        } else {
            uint32_t sg;
            F0 = scaled_mantissa(x[2 * i], e, sg);
            F1 = scaled_mantissa(x[2 * i + 1], e, sg);
        }
        uint32_t wi[S];
        digit_words(F0, h0, F1, h1, wi);
#pragma unroll
        for (int t = 0; t < S; t++) w[t][i] = wi[t];
    }
}

// C(r, j) = alpha * value (+ beta / C semantics)
__device__ __forceinline__ void store_out(const OzThinParams &p, double *cp, double v) {
    v *= p.alpha;
    if (p.semantics == GB_SEM_BLAS) {
        if (p.beta != 0.0) v = fma(p.beta, *cp, v);
    } else if (p.semantics == GB_SEM_SCALAR_BETA) {
        v = v + p.beta;
    } else {
        v = *cp + (v + p.beta);
    }
    *cp = v;
}

// The 16 values of row r in one 16-k box of X: [16 k][128 rows] (XCOLS) or
// 128 rows of 128 bytes with 16-byte chunks swizzled by row % 8.
template <bool XCOLS>
__device__ __forceinline__ void load_row16(const uint8_t *box, int r, double (&x)[16]) {
    if (XCOLS) {
        const double *xs = reinterpret_cast<const double *>(box);
#pragma unroll
        for (int k = 0; k < 16; k++) x[k] = xs[k * BM + r];
    } else {
        const uint8_t *rowp = box + r * 128;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const double2 v = *reinterpret_cast<const double2 *>(rowp + ((c ^ (r & 7)) << 4));
            x[2 * c] = v.x;
            x[2 * c + 1] = v.y;
        }
    }
}

// The 8 values k = 8h .. 8h+7 of row r in one 16-k box of X (layouts as
// load_row16).
template <bool XCOLS>
__device__ __forceinline__ void load_row8(const uint8_t *box, int r, int h, double (&x)[8]) {
    if (XCOLS) {
        const double *xs = reinterpret_cast<const double *>(box) + 8 * h * BM;
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = xs[k * BM + r];
    } else {
        const uint8_t *rowp = box + r * 128;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const double2 v = *reinterpret_cast<const double2 *>(rowp + (((4 * h + c) ^ (r & 7)) << 4));
            x[2 * c] = v.x;
            x[2 * c + 1] = v.y;
        }
    }
}


// X leading dimensions that TMA cannot describe (odd, or a base that is not
// 16-byte aligned): the producer warp copies k block kb of row tile rt with
// 8-byte cp.async into the layout the TMA boxes have (two 16-k boxes, SW128
// rows or [16 k][128 rows]), lane = k (row-major X: one row per instruction,
// 256 contiguous bytes) or lane = row (K-major X: 32 rows of one k), zeros
// outside X.
template <bool XCOLS>
__device__ __forceinline__ void copy_x_block(uint32_t st, const OzThinParams &p, int rt, int kb, int lane) {
    const int64_t r0 = (int64_t)rt * BM, k0 = (int64_t)kb * KB;
    const bool full_tile = r0 + BM <= p.rows && k0 + KB <= p.K;
    if (XCOLS) {   // k line k: rows r0 + 32q + lane, 256 contiguous bytes per q
        const double *src = p.X + k0 * p.ldx + r0 + lane;
        const uint32_t dst = st + (uint32_t)lane * 8;
        if (full_tile) {
#pragma unroll 4
            for (int k = 0; k < KB; k++, src += p.ldx) {
                const uint32_t d = dst + (uint32_t)((k / 16) * (XS / 2) + (k % 16) * BM * 8);
#pragma unroll
                for (int q = 0; q < BM / 32; q++) ptx::cp_async8(d + q * 256, src + 32 * q, 8u);
            }
        } else {
            for (int k = 0; k < KB; k++, src += p.ldx) {
                const uint32_t d = dst + (uint32_t)((k / 16) * (XS / 2) + (k % 16) * BM * 8);
                const bool kin = k0 + k < p.K;
#pragma unroll
                for (int q = 0; q < BM / 32; q++) {
                    const bool in = kin && r0 + 32 * q + lane < p.rows;
                    ptx::cp_async8(d + q * 256, in ? src + 32 * q : p.X, in ? 8u : 0u);
                }
            }
        }
    } else {       // row r: k0 + lane, 256 contiguous bytes per row; SW128 chunk (lane/2)%8 ^ r%8
        const double *src = p.X + r0 * p.ldx + k0 + lane;
        const int c = (lane % 16) / 2;
        const uint32_t dst = st + (uint32_t)((lane / 16) * (XS / 2) + (lane & 1) * 8);
        if (full_tile) {
            for (int r8 = 0; r8 < BM; r8 += 8) {
#pragma unroll
                for (int j = 0; j < 8; j++, src += p.ldx)
                    ptx::cp_async8(dst + (uint32_t)((r8 + j) * 128 + ((c ^ j) << 4)), src, 8u);
            }
        } else {
            const bool kin = k0 + lane < p.K;
            for (int r8 = 0; r8 < BM; r8 += 8) {
#pragma unroll
                for (int j = 0; j < 8; j++, src += p.ldx) {
                    const bool in = kin && r0 + r8 + j < p.rows;
                    ptx::cp_async8(dst + (uint32_t)((r8 + j) * 128 + ((c ^ j) << 4)), in ? src : p.X, in ? 8u : 0u);
                }
            }
        }
    }
}

template <bool XCOLS, bool CPA, int NG>
__global__ void __launch_bounds__(NT, 1)
    thin_oz_kernel(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmw, OzThinParams p) {
    constexpr int STAGES = Cfg<NG>::STAGES, STAGE = Cfg<NG>::STAGE, WS = Cfg<NG>::WS, PW = NG * NB;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *sring = smem + STAGES * STAGE;
    uint64_t *full = reinterpret_cast<uint64_t *>(sring + SSTAGES * XS);
    uint64_t *empty = full + STAGES;
    uint64_t *aready = empty + STAGES;     // [2] digit slots
    uint64_t *aempty = aready + 2;
    uint64_t *lfull = aempty + 2;          // [2] level sets (NG = 1: alternating; NG = 2: one per group)
    uint64_t *lempty = lfull + 2;
    uint64_t *sfull = lempty + 2;          // [SSTAGES] scan ring
    uint64_t *sempty = sfull + SSTAGES;
    uint64_t *xready = sempty + SSTAGES;   // [2] chunk exponents written
    // [2] chunk exponents read, by the converters (xfree_c) and by the drain (xfree_d): apart,
    // because the converters can run two chunks ahead of a drain held up in an epilogue, and
    // their arrivals for chunk c + 2 must not complete the phase of chunk c
    uint64_t *xfree_c = xready + 2;
    uint64_t *xfree_d = xfree_c + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(xfree_d + 2);
    int *exps = reinterpret_cast<int *>(reinterpret_cast<uint8_t *>(full) + BAR_BYTES);   // [2][BM]

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int nkb = (int)((p.K + KB - 1) / KB);
    const int units = p.rtiles * p.splits;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            ptx::mbar_init(&full[s], CPA ? 33 : 1);   // (the 32 copying lanes +) the W box's expect_tx
            ptx::mbar_init(&empty[s], 1 + NCONV);   // the MMA commit + the converter warps
        }
        for (int s = 0; s < SSTAGES; s++) {
            ptx::mbar_init(&sfull[s], CPA ? 32 : 1);
            ptx::mbar_init(&sempty[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            ptx::mbar_init(&aready[a], NCONV);
            ptx::mbar_init(&aempty[a], 1);
            ptx::mbar_init(&lfull[a], 1);
            ptx::mbar_init(&lempty[a], 4);
            ptx::mbar_init(&xready[a], 1);
            ptx::mbar_init(&xfree_c[a], NCONV);
            ptx::mbar_init(&xfree_d[a], 4);
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

    if (warp == 0 || warp == 14) {
        // producers: warp 0 the converter stages (X + W digits), warp 14 the scan ring; X by TMA
        // (lane 0) or, for leading dimensions TMA cannot take, by cp.async from all lanes
        const bool scan = warp == 14;
        const int nst = scan ? SSTAGES : STAGES;
        uint64_t *fb = scan ? sfull : full, *eb = scan ? sempty : empty;
        if (CPA || lane == 0) {
            int g = 0;
            bool go = true;
            for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
                const int rt = u / p.splits, sp = u - rt * p.splits;
                const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
                for (int kb = kb0; kb < kb1; kb++, g++) {
                    const int s = g % nst;
                    if (g >= nst && !ptx::mbar_wait(&eb[s], ((g / nst) & 1) ^ 1, p.err, scan ? 60 : 61)) {
                        go = false;
                        break;
                    }
                    uint8_t *st = scan ? sring + s * XS : smem + s * STAGE;
                    if (lane == 0 && !(CPA && scan)) {   // TMA bytes: X boxes (TMA loads) + the W digit box
                        ptx::mbar_arrive_expect_tx(&fb[s], (CPA ? 0 : XS) + (scan ? 0 : WS));
                        if (!CPA) {
#pragma unroll
                            for (int b = 0; b < 2; b++) {
                                if (XCOLS) ptx::tma_load_2d(st + b * (XS / 2), &tmx, &fb[s], rt * BM, kb * KB + 16 * b);
                                else ptx::tma_load_2d(st + b * (XS / 2), &tmx, &fb[s], kb * KB + 16 * b, rt * BM);
                            }
                        }
                        if (!scan) ptx::tma_load_2d(st + XS, &tmw, &fb[s], kb * KB, 0);
                    }
                    if (CPA) {
                        copy_x_block<XCOLS>(ptx::smem_u32(st), p, rt, kb, lane);
                        ptx::cp_async_mbar_arrive_noinc(&fb[s]);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            int g = 0, ch = 0;
            bool go = true;
            for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
                const int sp = u % p.splits;
                const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
                for (int c0 = kb0; c0 < kb1 && go; c0 += CHUNK_KB, ch++) {
                    const int c1 = min(kb1, c0 + CHUNK_KB);
                    const int use = NG == 1 ? (ch >> 1) : ch;   // earlier uses of this chunk's level sets
                    for (int kb = c0; kb < c1 && go; kb++, g++) {
                        const int s = g % STAGES, a = g & 1;
                        if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 63) ||
                            !ptx::mbar_wait(&aready[a], (g >> 1) & 1, p.err, 64)) {
                            go = false;
                            break;
                        }
                        ptx::tc_fence_after();
                        const uint32_t wst = ptx::smem_u32(smem + s * STAGE + XS);
                        const uint32_t slot = tmem + SLOT0 + (uint32_t)(a * SLOT_COLS);
                        // level sets: NG = 1 alternates two 128-column sets per chunk; NG = 2 has one
                        // 256-column set, the two groups' columns interleaved level by level
                        const int lb = NG == 1 ? (ch & 1) : 0;
                        if (kb == c0 && use >= 1) {   // the drain has read this level set's last chunk
                            if (!ptx::mbar_wait(&lempty[lb], (use & 1) ^ 1, p.err, 62)) {
                                go = false;
                                break;
                            }
                            ptx::tc_fence_after();
                        }
                        const uint32_t lv = tmem + (uint32_t)(lb * LV_COLS);
#pragma unroll
                        for (int kk = 0; kk < KB / 16; kk++) {
#pragma unroll
                            for (int t = 1; t <= S; t++) {
                                // W digits u = 9-t .. 1 of all NG groups: tile rows PW(t-1) .. 8PW-1,
                                // N = PW(9-t); the first MMA of a chunk (t = 1) writes every level column
                                const uint64_t bdesc = ptx::sdesc_kmajor_sw64(wst + (uint32_t)((t - 1) * PW * 64)) +
                                                       (uint64_t)((kk * 32) >> 4);
                                ptx::umma_f16_ta(lv, slot + (uint32_t)((t - 1) * 16 + kk * 8), bdesc,
                                                 ptx::idesc_bf16_f32(BM, PW * (S + 1 - t)),
                                                 (kb != c0 || kk != 0 || t != 1) ? 1u : 0u);
                            }
                        }
                        if (!go) break;
                        ptx::umma_commit(&empty[s]);
                        ptx::umma_commit(&aempty[a]);
                    }
                    if (go) ptx::umma_commit(&lfull[NG == 1 ? (ch & 1) : 0]);
                }
            }
        }
    } else if (warp < 2 + NCONV) {   // converters: thread = row q*32 + lane, one 16-k box each
        const int q = warp % 4, r = q * 32 + lane, b = (warp - 2) / 4;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int g = 0, ch = 0;
        bool go = true;
        for (int u = blockIdx.x; u < units && go; u += gridDim.x) {
            const int sp = u % p.splits;
            const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
            int e = 0;
            bool fast = true;
            for (int kb = kb0; kb < kb1; kb++, g++) {
                if ((kb - kb0) % CHUNK_KB == 0) {   // a new chunk: the row's exponent over it
                    const int xs = ch & 1;
                    if (!ptx::mbar_wait(&xready[xs], (ch >> 1) & 1, p.err, 68)) {
                        go = false;
                        break;
                    }
                    e = exps[xs * BM + r];
                    __syncwarp();
                    if (lane == 0) ptx::mbar_arrive(&xfree_c[xs]);
                    if (e == NO_EXP) e = 0;
                    fast = __all_sync(0xFFFFFFFFu, e >= -974);
                    ch++;
                }
                const int s = g % STAGES, a = g & 1;
                if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 65) ||
                    (g >= 2 && !ptx::mbar_wait(&aempty[a], ((g >> 1) & 1) ^ 1, p.err, 66))) {
                    go = false;
                    break;
                }
                ptx::tc_fence_after();
                const uint32_t slot = tmem + lane_off + SLOT0 + (uint32_t)(a * SLOT_COLS);
                double x[16];
                load_row16<XCOLS>(smem + s * STAGE + b * (XS / 2), r, x);
                uint32_t w[S][8];   // digit t, k pair i -> bf16x2
                if (fast) convert16<true>(x, e, w);
                else convert16<false>(x, e, w);
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
    } else if (warp < 14) {  // drain chunk c, epilogue: thread = row q*32 + lane of the tile
        const int q = warp % 4, r = q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        Walk dw;
        dw.first(p, nkb);
        bool go = true;
        double acc[NG * NB];
#pragma unroll
        for (int j = 0; j < NG * NB; j++) acc[j] = 0.0;
        int eref = NO_EXP;   // the row's largest chunk exponent so far: acc is in units of 2^eref
        bool nf = false;     // the row holds an Inf / NaN
        for (int ch = 0; go && dw.u < units; ch++) {
            const int xs = ch & 1;
            if (!ptx::mbar_wait(&xready[xs], (ch >> 1) & 1, p.err, 70)) break;
            const int ec = exps[xs * BM + r];
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&xfree_d[xs]);
            nf |= ec == kNonFiniteLineExp;
            if (ec != NO_EXP) {
                if (eref == NO_EXP) {
                    eref = ec;
                } else if (ec > eref) {
#pragma unroll
                    for (int j = 0; j < NG * NB; j++) acc[j] = mul_pow2(acc[j], eref - ec);
                    eref = ec;
                }
            }
            // T = sum_L S_L 2^(6(9-L)) exactly in 64-bit integers (|S_L| < (L-1) 256 63^2, so
            // |T| < 2^62.1), then one rounding to FP64: sum_L S_L 2^-6L = T 2^-54
            const double sc = pow2_or_zero(ec == NO_EXP ? -100000 : ec - eref - 54);
            const int use = NG == 1 ? (ch >> 1) : ch;
            const int lb = NG == 1 ? (ch & 1) : 0;
            if (!ptx::mbar_wait(&lfull[lb], use & 1, p.err, 67)) break;
            ptx::tc_fence_after();
#pragma unroll
            for (int gr = 0; gr < NG; gr++) {
#pragma unroll
                for (int h = 0; h < NB / 4; h++) {   // four columns at a time, the 8 level loads in flight together
                    uint32_t v[S][4];
#pragma unroll
                    for (int L = 2; L <= S + 1; L++)
                        ptx::tmem_ld_32x32b_x4(tmem + lane_off +
                                                   (uint32_t)(lb * LV_COLS + (S + 1 - L) * PW + gr * NB + 4 * h),
                                               v[L - 2]);
                    ptx::tmem_ld_wait();
                    if (gr == NG - 1 && h == NB / 4 - 1) {   // the whole level set is in registers: back to the MMA
                        ptx::tc_fence_before();
                        __syncwarp();
                        if (lane == 0) ptx::mbar_arrive(&lempty[lb]);
                    }
                    long long T[4] = {0, 0, 0, 0};
#pragma unroll
                    for (int L = 0; L < S; L++)
#pragma unroll
                        for (int j = 0; j < 4; j++) T[j] = T[j] * 64 + (long long)__float2int_rn(__uint_as_float(v[L][j]));
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[gr * NB + 4 * h + j] = fma((double)T[j], sc, acc[gr * NB + 4 * h + j]);
                }
            }
            if (!go) break;
            if (dw.last()) {   // the unit's sums are complete
                const int rt = dw.u / p.splits, sp = dw.u - rt * p.splits;
                const int64_t row = (int64_t)rt * BM + r;
                if (row < p.rows) {
                    const int er = eref == NO_EXP ? 0 : eref;
                    if (p.splits > 1) {
                        double *pp = p.part + ((int64_t)sp * p.rows + row) * p.pw;
#pragma unroll
                        for (int j = 0; j < NG * NB; j++)
                            if (j < p.n) pp[j] = mul_pow2(acc[j], er + __ldg(p.fcol + j));
                        if (nf) p.nfrow[row] = 1;
                    } else {
                        double *cr = p.C + row * p.cs_r;
#pragma unroll
                        for (int j = 0; j < NG * NB; j++) {
                            if (j >= p.n) break;
                            const int fc = __ldg(p.fcol + j);
                            if (!nf && fc != kNonFiniteLineExp)
                                store_out(p, cr + (int64_t)j * p.cs_c, mul_pow2(acc[j], er + fc));
                        }
#pragma unroll 1
                        for (int j = 0; j < p.n; j++)   // a row or column that holds an Inf / NaN
                            if (nf || __ldg(p.fcol + j) == kNonFiniteLineExp)
                                store_out(p, cr + (int64_t)j * p.cs_c,
                                          native_dot(p.X, p.ldx, p.tx, row, p.W, p.ldw, p.tw, (int64_t)p.j0 + j, p.K));
                    }
                }
#pragma unroll
                for (int j = 0; j < NG * NB; j++) acc[j] = 0.0;
                eref = NO_EXP;
                nf = false;
            }
            dw.next(p, nkb);
        }
    } else if (warp == 15) {   // scan: chunk c+1 while chunk c converts; lane = rows lane + 32i
        Walk sw;
        sw.first(p, nkb);
        int sg = 0;
        for (int sch = 0; sw.u < units; sch++) {
            // the largest |high word| gives the exponent unless it is subnormal; then the bit
            // length of the largest |x| is that of the OR of all (high, low) words
            uint32_t mx[4] = {0, 0, 0, 0}, lor[4] = {0, 0, 0, 0};
            // NG = 2 (slower chunks): start once chunk sch - 1 is being converted, at most one
            // chunk ahead, so that the conversion's re-read of this chunk still finds it in L2
            // (two chunks ahead doubled the DRAM reads); NG = 1 keeps the scan two ahead
            const int lag = NG == 2 ? 1 : 2;
            if (sch >= lag) {
                const int ps = (sch - lag) & 1, ph = ((sch - lag) >> 1) & 1;
                if (!ptx::mbar_wait(&xfree_c[ps], ph, p.err, 71) || !ptx::mbar_wait(&xfree_d[ps], ph, p.err, 72)) break;
            }
            bool go = true;
            for (int kb = sw.c0; kb < sw.c1(); kb++, sg++) {
                const int s = sg % SSTAGES;
                if (!ptx::mbar_wait(&sfull[s], (sg / SSTAGES) & 1, p.err, 69)) {
                    go = false;
                    break;
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
#pragma unroll
                    for (int bh = 0; bh < 4; bh++) {
                        double x[8];
                        load_row8<XCOLS>(sring + s * XS + (bh >> 1) * (XS / 2), lane + 32 * i, bh & 1, x);
#pragma unroll
                        for (int k = 0; k < 8; k += 2) {
                            const uint32_t h0 = (uint32_t)__double2hiint(x[k]) & 0x7FFFFFFFu;
                            const uint32_t h1 = (uint32_t)__double2hiint(x[k + 1]) & 0x7FFFFFFFu;
                            mx[i] = __vimax3_u32(mx[i], h0, h1);
                            lor[i] |= (uint32_t)__double2loint(x[k]) | (uint32_t)__double2loint(x[k + 1]);
                        }
                    }
                }
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&sempty[s]);
            }
            if (!go) break;
            const int xs = sch & 1;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                int e;
                if (mx[i] >> 20) e = (int)(mx[i] >> 20) - 1022;                      // normal, Inf, NaN
                else if (mx[i]) e = 64 - __clz(mx[i]) - 1074;                        // subnormal, high word set
                else e = lor[i] ? 32 - __clz(lor[i]) - 1074 : NO_EXP;                // tiny subnormal, or zeros
                exps[xs * BM + lane + 32 * i] = e;
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&xready[xs]);
            sw.next(p, nkb);
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// Split-K: sum the parts (already scaled) in order, then the epilogue; a
// row or column holding an Inf / NaN gets the plain dot product.
__global__ void thin_oz_reduce_kernel(OzThinParams p) {
    const int64_t total = p.rows * p.n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / p.n;
        const int j = (int)(e - r * p.n);
        double s = 0.0;
        if (p.nfrow[r] || __ldg(p.fcol + j) == kNonFiniteLineExp) {
            s = native_dot(p.X, p.ldx, p.tx, r, p.W, p.ldw, p.tw, (int64_t)p.j0 + j, p.K);
        } else {
            for (int sp = 0; sp < p.splits; sp++) s += p.part[((int64_t)sp * p.rows + r) * p.pw + j];
        }
        store_out(p, p.C + r * p.cs_r + (int64_t)j * p.cs_c, s);
    }
}

// Digits of W columns j0 .. j0+pw-1 (logical K x n; tw: stored n x K),
// relative to the column exponents: out[(8-u)*pw + jp][k] for column j0 + jp
// and u = 1..8 (the least significant digit first, the pass's columns within
// a digit), K-major, kp columns, zero beyond n and K.
__global__ void wdigits_kernel(const double *__restrict__ W, int64_t ldw, int tw, int n, int j0, int pw, int64_t K,
                               int64_t kp, const int *__restrict__ fcol, unsigned short *__restrict__ out) {
    const int64_t total = (int64_t)pw * kp;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int jp = (int)(e / kp);
        const int64_t k = e - (int64_t)jp * kp;
        const int j = j0 + jp;
        double x = 0.0;
        int f = 0;
        if (j < n && k < K) {
            x = tw ? W[(int64_t)j * ldw + k] : W[k * ldw + j];
            f = fcol[jp];
        }
        uint32_t sg;
        const uint64_t F = scaled_mantissa(x, f, sg);
#pragma unroll
        for (int u = 1; u <= S; u++) {
            const uint32_t d = digit_of(F, u);
            const unsigned short h =
                d ? (unsigned short)(__bfloat16_as_ushort(__float2bfloat16_rn(small_int_to_float(d))) | (sg << 15))
                  : 0;
            out[((int64_t)(S - u) * pw + jp) * kp + k] = h;
        }
    }
}

template <bool XCOLS, bool CPA, int NG>
cudaError_t set_smem() {
    return cudaFuncSetAttribute(thin_oz_kernel<XCOLS, CPA, NG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                Cfg<NG>::SMEM);
}

}  // namespace thin_oz
}  // namespace

// FP64 skinny product through digits on the tensor cores.  X rows x K
// (tx: stored K x rows), W K x n (tw: stored n x K), n <= 64 in passes of up
// to 32 columns, C(r, j) at C[r*cs_r + j*cs_c].  Scratch: `ws` of
// thin_oz_workspace_bytes() bytes.
size_t thin_oz_workspace_bytes(int64_t rows, int64_t K, int n, int splits) {
    const int64_t kp = ceil_div(K, thin_oz::KB) * thin_oz::KB;
    size_t b = (size_t)(rows + 64) * 4 + 256;                                // row flags (+ column exponents)
    b += (size_t)thin_oz::S * 2 * thin_oz::NB * kp * 2 + 256;              // W digit slices of one pass
    if (splits > 1) b += (size_t)splits * rows * 2 * thin_oz::NB * 8;      // split-K parts
    (void)n;
    return b;
}

bool thin_oz_eligible(int tx, int64_t ldx, const void *X, int64_t rows, int64_t K) {
    const char *e = getenv("GB_SKINNY_OZ");   // "0": native FP64 kernels (measurement)
    if (e && e[0] == '0') return false;
    (void)tx;
    (void)ldx;
    return K >= 64 && rows < (int64_t(1) << 31) && K < (int64_t(1) << 30) && (uintptr_t)X % 8 == 0;
}

gb_status launch_thin_oz(int64_t rows, int64_t K, const double *X, int64_t ldx, int tx, const double *W, int64_t ldw,
                         int tw, int n, double *C, int64_t cs_r, int64_t cs_c, double alpha, double beta,
                         int semantics, int splits, int64_t kchunk, void *ws, cudaStream_t st) {
    using namespace thin_oz;
    const int64_t kp = ceil_div(K, KB) * KB;
    uint8_t *w8 = (uint8_t *)ws;   // row flags, column exponents, W digits of a pass, split-K parts
    int *nfrow = (int *)w8;    // split-K: rows holding an Inf / NaN
    int *fcol = nfrow + rows;  // up to 64 columns
    size_t off = ((size_t)(rows + 64) * 4 + 255) / 256 * 256;
    unsigned short *wd = (unsigned short *)(w8 + off);
    off += ((size_t)S * 2 * NB * kp * 2 + 255) / 256 * 256;
    double *part = splits > 1 ? (double *)(w8 + off) : nullptr;
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "skinny: no device error word");

    gb_status s = ozaki_line_exponents(W, ldw, tw == 0, n, K, fcol, st);
    if (s != GB_OK) return s;
    if (splits > 1) GB_CUDA_TRY(cudaMemsetAsync(nfrow, 0, (size_t)rows * 4, st));

    // X through TMA when its rows (or k lines) start on 16-byte boundaries, else by cp.async
    const char *force = getenv("GB_SKINNY_OZ_CPASYNC");   // "1": the cp.async loader for any X (tests)
    const bool cpa = ldx % 2 != 0 || (uintptr_t)X % 16 != 0 || (force && force[0] == '1');
    CUtensorMap tx_map, tw_map[2];   // W digit boxes of one or two column groups
    const bool okw =
        make_tmap_bf16(&tw_map[0], wd, (uint64_t)kp, (uint64_t)2 * S * NB, (uint64_t)kp * 2, KB, S * NB, 64) &&
        make_tmap_bf16(&tw_map[1], wd, (uint64_t)kp, (uint64_t)2 * S * NB, (uint64_t)kp * 2, KB, 2 * S * NB, 64);
    bool okx = true;
    if (cpa) tx_map = tw_map[0];   // unused
    else if (tx) okx = make_tmap_f64(&tx_map, X, (uint64_t)rows, (uint64_t)K, (uint64_t)ldx * 8, BM, 16, false);
    else okx = make_tmap_f64(&tx_map, X, (uint64_t)K, (uint64_t)rows, (uint64_t)ldx * 8, 16, BM, true);
    if (!okx || !okw) return set_status(GB_ERR_CUDA, "skinny: cuTensorMapEncodeTiled failed");

    static std::atomic<uint64_t> attr{0};
    if (device_setup_needed(attr)) {
        GB_CUDA_TRY((set_smem<false, false, 1>()));
        GB_CUDA_TRY((set_smem<true, false, 1>()));
        GB_CUDA_TRY((set_smem<false, true, 1>()));
        GB_CUDA_TRY((set_smem<true, true, 1>()));
        GB_CUDA_TRY((set_smem<false, false, 2>()));
        GB_CUDA_TRY((set_smem<true, false, 2>()));
        GB_CUDA_TRY((set_smem<false, true, 2>()));
        GB_CUDA_TRY((set_smem<true, true, 2>()));
        device_setup_done(attr);
    }
    const int rtiles = (int)ceil_div(rows, BM);
    const int units = rtiles * splits;
    const int grid = units < sm_count() ? units : sm_count();
    for (int j0 = 0; j0 < n;) {   // up to 32 columns of W per pass over X
        const int ng = n - j0 > NB ? 2 : 1;
        const int pw = ng * NB, nc = n - j0 < pw ? n - j0 : pw;
        const int64_t wtot = (int64_t)pw * kp;
        const int blocks = (int)(ceil_div(wtot, 256) < 2 * sm_count() ? ceil_div(wtot, 256) : 2 * sm_count());
        wdigits_kernel<<<blocks, 256, 0, st>>>(W, ldw, tw, n, j0, pw, K, kp, fcol + j0, wd);
        GB_LAUNCH_CHECK("wdigits_kernel");
        OzThinParams p{rows, K, nc, splits, (int)(kchunk / KB), rtiles, pw,
                       C + j0 * cs_c, cs_r, cs_c, alpha, beta, semantics, part, nfrow, fcol + j0, err,
                       X, W, ldx, ldw, tx, tw, j0};
        const CUtensorMap &twm = tw_map[ng - 1];
        if (ng == 1) {
            const int sm = Cfg<1>::SMEM;
            if (tx && cpa) thin_oz_kernel<true, true, 1><<<grid, NT, sm, st>>>(tx_map, twm, p);
            else if (tx) thin_oz_kernel<true, false, 1><<<grid, NT, sm, st>>>(tx_map, twm, p);
            else if (cpa) thin_oz_kernel<false, true, 1><<<grid, NT, sm, st>>>(tx_map, twm, p);
            else thin_oz_kernel<false, false, 1><<<grid, NT, sm, st>>>(tx_map, twm, p);
        } else {
            const int sm = Cfg<2>::SMEM;
            if (tx && cpa) thin_oz_kernel<true, true, 2><<<grid, NT, sm, st>>>(tx_map, twm, p);
            else if (tx) thin_oz_kernel<true, false, 2><<<grid, NT, sm, st>>>(tx_map, twm, p);
            else if (cpa) thin_oz_kernel<false, true, 2><<<grid, NT, sm, st>>>(tx_map, twm, p);
            else thin_oz_kernel<false, false, 2><<<grid, NT, sm, st>>>(tx_map, twm, p);
        }
        GB_LAUNCH_CHECK("thin_oz_kernel");
        if (splits > 1) {
            const int rb = (int)(ceil_div(rows * nc, 256) < 4 * sm_count() ? ceil_div(rows * nc, 256) : 4 * sm_count());
            thin_oz_reduce_kernel<<<rb, 256, 0, st>>>(p);
            GB_LAUNCH_CHECK("thin_oz_reduce_kernel");
        }
        j0 += pw;
    }
    return ok();
}

}  // namespace gb
