// gemm_ozaki.cu -- DGEMM from exact integer slices on the tcgen05 tensor cores
// (Ozaki scheme: Ozaki, Ogita, Oishi & Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012; integer-slice form as in
// Ootomo, Ozaki & Yokota, "DGEMM on integer matrix multiplication unit",
// IJHPCA 2024).  Precision form of the reference's DGEMM
// (dgemm_release_V1.1/device_code/dgemm_kernel.c:1994-3170); it has no
// counterpart in the reference.
//
// Each row i of op(A) is scaled by 2^-e_i (e_i: max_k |a_ik| < 2^e_i) and
// written as s balanced base-256 digits, a_ik = 2^(e_i+1) * sum_t v_ikt 2^-8t
// (+ a remainder of at most half of 2^(e_i+1-8s)), v in [-128, 127] (the leading digit
// in [-128, 128]); columns of op(B) likewise with exponents f_j and digits w.
// Then
//     C_ij ~= 2^(e_i+f_j+2) sum_{t+u <= s+1} 2^-8(t+u) (V_t W_u^T)_ij .
// The digits are integers that BF16 holds exactly (|v| <= 128), so each slice
// product runs on tcgen05.mma kind::f16 with an FP32 accumulator in TMEM, and
// every partial sum of a 1024-long K chunk is an integer of magnitude at most
// 1024*128^2 = 2^24: exact.  Eight bits per slice (balanced digits keep the
// products within 2^14 although they carry a full byte) give FP64-level
// results with 7 slices (28 slice products) and no worse than native FP64
// with 8 (36, the default).  Chunk sums are added exactly in int32 registers (up to 127 chunks),
// and FP64 appears only in the per-pair scaled sum kept in TMEM and in the
// final 2^(e_i+f_j), alpha, beta epilogue.  (sm_103a has no kind::i8 MMA, so
// the INT8 products are carried in BF16; products and sums stay exact.)
//
// Kernels: row/column exponents (integer max of |x| bit patterns), digit
// extraction (integer shifts of the FP64 mantissa; the transpose modes are
// absorbed here, slices are written K-major), and a persistent GEMM: one CTA
// per SM over 128 x 128 C tiles, per tile a loop over slice pairs and K
// chunks; warp 0 issues TMA (one digit tile of V_t and one of W_u per 64-wide
// K block), warp 1 issues the MMAs into one of two FP32 accumulators
// (alternating per chunk), warps 2-5 drain them into int32 registers and the
// FP64 sum in TMEM, and write C.
#include <cuda.h>
#include <limits.h>
#include <cuda_bf16.h>

#include "gb_common.cuh"
#include "sm100_ptx.cuh"

namespace gb {

bool make_tmap_bf16(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                    uint32_t box_inner, uint32_t box_outer, int swizzle_bytes);

int ozaki_pick_slices(double target_err, int64_t K) {
    // Each input is truncated at 2^(1-8s) of its row (column) maximum, so a
    // product term errs by at most ~2^(2-8s) |a||b|; FP64's own rounding is
    // u = 2^-53 per term, and both grow like sqrt(K) over a dot product.
    // target_err 0 (FP64-equivalent): no worse than native FP64, s = 8
    // (measured on 8192^3 with entries u*2^e, e in [-20, 20]: 8.3e-19 against
    // native 7.5e-18; s = 7 measured 7.56e-18, a little worse than native).
    // A target: the smallest s with 2^(2-8s) sqrt(K) * 4 <= target.
    if (target_err <= 0) return 8;
    double logk = 0;
    for (int64_t k = K; k > 1; k >>= 1) logk += 0.5;
    for (int s = 2; s <= 9; s++)
        if (2.0 - 8.0 * s + logk + 2.0 <= __builtin_log2(target_err)) return s;
    return 9;
}

namespace {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 6, GROUP_M = 8;
constexpr int KCHUNK_BLOCKS = 16;              // 1024-long exact FP32 chunk
constexpr int MAX_CHUNKS_INT32 = 127;          // chunk sums per int32 accumulator
constexpr int MAXS = 9, MAXPAIRS = MAXS * (MAXS + 1) / 2;
constexpr int TILE_BYTES = BM * BK * 2;        // 16 KB (BM == BN)
constexpr int STAGE_BYTES = 2 * TILE_BYTES;
constexpr int EPI_BYTES = 4 * 32 * 33 * 8;     // per-warp 32 x 32 FP64 staging
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EPI_BYTES + 1024 + 256;
static_assert(SMEM_BYTES <= 232448, "shared memory");
constexpr int NT = 192;
constexpr uint32_t TMEM_COLS = 512;            // [0,256): two FP32 accumulators, [256,512): FP64 sum

// ------------------------------------------------------------- exponents
// (exp_of_maxbits: the line exponent from the maximum |x| bit pattern)

// one warp per line of `len` contiguous elements
__global__ void maxexp_contig_kernel(const double *__restrict__ X, int64_t ld, int64_t lines, int64_t len,
                                     int *__restrict__ e) {
    const int64_t line = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (line >= lines) return;
    unsigned long long mb = 0;
    const unsigned long long *p = reinterpret_cast<const unsigned long long *>(X + line * ld);
    for (int64_t k = lane; k < len; k += 32) {
        unsigned long long b = __ldg(p + k) & 0x7FFFFFFFFFFFFFFFull;
        mb = b > mb ? b : mb;
    }
    for (int o = 16; o; o >>= 1) {
        unsigned long long v = __shfl_xor_sync(0xffffffffu, mb, o);
        mb = v > mb ? v : mb;
    }
    if (lane == 0) e[line] = exp_of_maxbits(mb);
}

// Column exponents of a len x cols storage (rows strided by ld), in three
// small kernels: e[] = INT_MIN; each block reduces 32 consecutive columns
// (lane = column, coalesced) over kpb rows and raises e[col] to the
// exponent of its maximum (exponents are monotone in |x|, so the maximum of
// the partial exponents is the exponent of the maximum; an all-zero part
// contributes INT_MIN); INT_MIN (an all-zero column) -> 0.
__global__ void exp_init_kernel(int *__restrict__ e, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        e[i] = INT_MIN;
}

__global__ void __launch_bounds__(256) maxexp_strided_kernel(const double *__restrict__ X, int64_t ld, int64_t cols,
                                                             int64_t len, int64_t kpb, int *__restrict__ e) {
    __shared__ unsigned long long part[8][32];
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    const int64_t j = (int64_t)blockIdx.x * 32 + lane;
    const int64_t k0 = (int64_t)blockIdx.y * kpb;
    unsigned long long mb = 0;
    if (j < cols) {
        const unsigned long long *p = reinterpret_cast<const unsigned long long *>(X);
        const int64_t k1 = k0 + kpb < len ? k0 + kpb : len;
#pragma unroll 8
        for (int64_t k = k0 + w; k < k1; k += 8) {
            const unsigned long long b = __ldg(p + k * ld + j) & 0x7FFFFFFFFFFFFFFFull;
            mb = b > mb ? b : mb;
        }
    }
    part[w][lane] = mb;
    __syncthreads();
    if (w == 0 && j < cols) {
#pragma unroll
        for (int i = 1; i < 8; i++) mb = part[i][lane] > mb ? part[i][lane] : mb;
        if (mb != 0) atomicMax(e + j, exp_of_maxbits(mb));
    }
}

__global__ void exp_finish_kernel(int *__restrict__ e, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (e[i] == INT_MIN) e[i] = 0;
}

static void launch_maxexp_strided(const double *X, int64_t ld, int64_t cols, int64_t len, int *e, cudaStream_t st) {
    const unsigned nb = (unsigned)(ceil_div(cols, 256) < 4096 ? ceil_div(cols, 256) : 4096);
    exp_init_kernel<<<nb, 256, 0, st>>>(e, cols);
    int64_t kpb = 256;   // rows per block; more when len would need over 65535 blocks in y
    while (ceil_div(len, kpb) > 65535) kpb *= 2;
    dim3 grid((unsigned)ceil_div(cols, 32), (unsigned)ceil_div(len, kpb));
    maxexp_strided_kernel<<<grid, 256, 0, st>>>(X, ld, cols, len, kpb, e);
    exp_finish_kernel<<<nb, 256, 0, st>>>(e, cols);
}

// ---------------------------------------------------------------- digits
// s balanced base-256 digits of x (|x| < 2^e): N = +-round(|x| 2^(8s-1-e))
// (to nearest: the representation error is half a unit of the last digit
// either way, where truncation erred up to a whole unit toward zero),
// |N| <= 2^(8s-1), cut from the least significant digit up (d = N mod 256 in
// [-128, 127], N = (N - d) / 256), so x ~= 2^(e+1) sum_t d_t 2^-8t; the
// leading digit is in [-128, 128].  Written as BF16, most significant first.
__device__ __forceinline__ void digits(double x, int e, int s, unsigned short *out, int64_t stride) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7FF);
    unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    int ex;
    if (E == 0) {
        ex = -1074;
    } else {
        m |= 1ull << 52;
        ex = E - 1075;
    }
    const int shift = ex + 8 * s - 1 - e;   // F = m * 2^shift <= 2^(8s-1) <= 2^71, rounded to nearest
    unsigned __int128 F = 0;
    if (m != 0 && shift > -64) {
        if (shift >= 0) {
            F = (unsigned __int128)m << shift;
        } else {   // half a unit of the last digit added first: the dropped part errs both ways
            const int rs = -shift;
            F = (unsigned __int128)((m + (1ull << (rs - 1))) >> rs);
        }
    }
    __int128 N = (b >> 63) ? -(__int128)F : (__int128)F;
    for (int t = s; t >= 1; t--) {
        const int d = (int)(((long long)N + 128) & 255) - 128;
        N = (N - d) >> 8;
        const int v = t == 1 ? d + 256 * (int)N : d;   // the leading digit takes what is left (|v| <= 128)
        const unsigned short h = v ? __bfloat16_as_ushort(__float2bfloat16_rn((float)v)) : 0;
        out[(int64_t)(t - 1) * stride] = h;
    }
}

// out: s slices of rows_p x kp (K-major).  Source element (r, k):
// trans ? X[k*ldx + r] : X[r*ldx + k]; padding rows / columns are zero.
__global__ void __launch_bounds__(256) slice_kernel(const double *__restrict__ X, int64_t ldx, int trans, int64_t rows,
                                                    int64_t K, int64_t rows_p, int64_t kp, const int *__restrict__ e,
                                                    int s, unsigned short *__restrict__ out) {
    __shared__ double tile[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
#pragma unroll
    for (int i = 0; i < 32; i += 8) {
        double v = 0.0;
        if (trans) {
            int64_t k = k0 + ty + i, r = r0 + tx;
            if (k < K && r < rows) v = X[k * ldx + r];
            tile[ty + i][tx] = v;
        } else {
            int64_t r = r0 + ty + i, k = k0 + tx;
            if (k < K && r < rows) v = X[r * ldx + k];
            tile[tx][ty + i] = v;
        }
    }
    __syncthreads();
    const int64_t stride = rows_p * kp;
#pragma unroll
    for (int i = 0; i < 32; i += 8) {
        int64_t r = r0 + ty + i, k = k0 + tx;
        if (r < rows_p && k < kp) digits(tile[tx][ty + i], r < rows ? e[r] : 0, s, out + r * kp + k, stride);
    }
}

// ------------------------------------------------------------------ gemm
struct OzParams {
    double *C;
    int64_t M, N, ldc;
    double alpha, beta;
    int semantics;
    int num_kb;                    // K blocks of 64
    int tiles_m, tiles_n;
    int64_t mp, np;                // padded rows of one V / W slice
    int npairs;
    signed char pt[MAXPAIRS], pu[MAXPAIRS];   // 1-based digit indices per pair
    const int *erow, *fcol;
    int *err;
    // operands, for the outputs that a non-finite row or column reaches
    const double *A, *B;
    int64_t lda, ldb, K;
    int ta, tb;
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
    ozaki_gemm_kernel(const __grid_constant__ CUtensorMap tmV, const __grid_constant__ CUtensorMap tmW, OzParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    double *epi = reinterpret_cast<double *>(smem + STAGES * STAGE_BYTES);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES + EPI_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;
    uint64_t *acc_empty = acc_full + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int num_tiles = p.tiles_m * p.tiles_n;
    const int nchunks = (p.num_kb + KCHUNK_BLOCKS - 1) / KCHUNK_BLOCKS;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            ptx::mbar_init(&acc_full[b], 1);
            ptx::mbar_init(&acc_empty[b], 4);
        }
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&tmV);
        ptx::tma_prefetch_desc(&tmW);
    }
    if (warp == 1) ptx::tmem_alloc(tmem_slot, TMEM_COLS);
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {   // TMA producer: per tile, per pair, every K block
            int kbg = 0;
            bool go = true;
            for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
                int tm, tn;
                tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
                for (int q = 0; q < p.npairs && go; q++) {
                    const int vrow = (int)((p.pt[q] - 1) * p.mp + (int64_t)tm * BM);
                    const int wrow = (int)((p.pu[q] - 1) * p.np + (int64_t)tn * BN);
                    for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
                        const int s = kbg % STAGES;
                        if (kbg >= STAGES && !ptx::mbar_wait(&empty[s], ((kbg / STAGES) & 1) ^ 1, p.err, 11)) {
                            go = false;
                            break;
                        }
                        uint8_t *st = smem + s * STAGE_BYTES;
                        ptx::mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
                        ptx::tma_load_2d(st, &tmV, &full[s], kb * BK, vrow);
                        ptx::tma_load_2d(st + TILE_BYTES, &tmW, &full[s], kb * BK, wrow);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer: one accumulator per K chunk of a pair
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, BN);
            int kbg = 0, gi = 0;
            bool go = true;
            for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
                for (int q = 0; q < p.npairs && go; q++) {
                    for (int c = 0; c < nchunks && go; c++, gi++) {
                        const int b = gi & 1;
                        if (gi >= 2 && !ptx::mbar_wait(&acc_empty[b], ((gi >> 1) & 1) ^ 1, p.err, 12)) {
                            go = false;
                            break;
                        }
                        ptx::tc_fence_after();
                        const uint32_t acc = tmem + (uint32_t)(b * BN);
                        const int kb_end = min(p.num_kb, (c + 1) * KCHUNK_BLOCKS);
                        for (int kb = c * KCHUNK_BLOCKS; kb < kb_end; kb++, kbg++) {
                            const int s = kbg % STAGES;
                            if (!ptx::mbar_wait(&full[s], (kbg / STAGES) & 1, p.err, 13)) {
                                go = false;
                                break;
                            }
                            ptx::tc_fence_after();
                            const uint32_t st = ptx::smem_u32(smem + s * STAGE_BYTES);
                            const uint64_t vd = ptx::sdesc_kmajor_sw128(st);
                            const uint64_t wd = ptx::sdesc_kmajor_sw128(st + TILE_BYTES);
#pragma unroll
                            for (int k = 0; k < BK / 16; k++) {
                                const uint64_t dk = (uint64_t)((k * 32) >> 4);
                                ptx::umma_f16(acc, vd + dk, wd + dk, idesc, (kb != c * KCHUNK_BLOCKS) || (k != 0));
                            }
                            ptx::umma_commit(&empty[s]);
                        }
                        if (go) ptx::umma_commit(&acc_full[b]);
                    }
                }
            }
        }
    } else {               // epilogue warps 2..5: TMEM lane quarter q = warp % 4
        const int q = warp % 4;
        double *stage = epi + q * 32 * 33;
        const uint32_t lane_base = (uint32_t)(q * 32) << 16;
        const uint32_t tot = tmem + 256u + lane_base;   // FP64 sum: element j at columns 2j, 2j+1
        int gi = 0;
        bool go = true;
        for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
            int tm, tn;
            tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
            bool first_flush = true;
            // exact int32 sums of the chunk sums of consecutive pairs on one diagonal t + u (one
            // scale): one FP64 flush per diagonal, or after MAX_CHUNKS_INT32 chunk sums
            int iacc[BN];
#pragma unroll
            for (int j = 0; j < BN; j++) iacc[j] = 0;
            int nacc = 0;
            for (int qq = 0; qq < p.npairs && go; qq++) {
                const int lev = p.pt[qq] + p.pu[qq];
                const bool lev_ends = qq == p.npairs - 1 || p.pt[qq + 1] + p.pu[qq + 1] != lev;
                const double scale = __longlong_as_double((long long)(1023 + 2 - 8 * lev) << 52);
                for (int c = 0; c < nchunks; c++, gi++) {
                    const int b = gi & 1;
                    if (!ptx::mbar_wait(&acc_full[b], (gi >> 1) & 1, p.err, 14)) { go = false; break; }
                    ptx::tc_fence_after();
#pragma unroll
                    for (int cb = 0; cb < BN / 32; cb++) {
                        uint32_t r[32];
                        ptx::tmem_ld_32x32b_x32(tmem + (uint32_t)(b * BN) + lane_base + (uint32_t)(cb * 32), r);
                        ptx::tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 32; j++) iacc[cb * 32 + j] += __float2int_rn(__uint_as_float(r[j]));
                    }
                    ptx::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) ptx::mbar_arrive(&acc_empty[b]);
                    const bool flush = (c == nchunks - 1 && lev_ends) || ++nacc == MAX_CHUNKS_INT32;
                    if (flush) {   // FP64 sum += 2^(2-8(t+u)) * iacc (exact scaling, one rounding)
                        nacc = 0;
#pragma unroll
                        for (int cb = 0; cb < (2 * BN) / 32; cb++) {
                            uint32_t r[32];
                            if (!first_flush) {
                                ptx::tmem_ld_32x32b_x32(tot + (uint32_t)(cb * 32), r);
                                ptx::tmem_ld_wait();
                            }
#pragma unroll
                            for (int j = 0; j < 16; j++) {
                                double v = first_flush ? 0.0 : __hiloint2double((int)r[2 * j + 1], (int)r[2 * j]);
                                v = fma((double)iacc[cb * 16 + j], scale, v);
                                r[2 * j] = (uint32_t)__double2loint(v);
                                r[2 * j + 1] = (uint32_t)__double2hiint(v);
                                iacc[cb * 16 + j] = 0;
                            }
                            ptx::tmem_st_32x32b_x32(tot + (uint32_t)(cb * 32), r);
                        }
                        ptx::tmem_st_wait();
                        first_flush = false;
                    }
                }
            }
            if (!go) break;
            // C = alpha * 2^(e_i + f_j) * sum (+ beta ...), staged for row-contiguous stores
            const int64_t row0 = (int64_t)tm * BM + q * 32;
            const int64_t n0 = (int64_t)tn * BN;
            const int64_t myrow = row0 + lane;
            const int erow = myrow < p.M ? p.erow[myrow] : 0;
            for (int cb = 0; cb < BN / 32; cb++) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    uint32_t r[32];
                    ptx::tmem_ld_32x32b_x32(tot + (uint32_t)(cb * 64 + h * 32), r);
                    ptx::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        stage[lane * 33 + h * 16 + j] = mul_pow2(__hiloint2double((int)r[2 * j + 1], (int)r[2 * j]), erow);
                }
                __syncwarp();
                const int64_t col = n0 + cb * 32 + lane;
                if (col < p.N) {
                    const int fc = p.fcol[col];
                    const int rows = (p.M - row0) < 32 ? (int)(p.M - row0) : 32;
                    const bool needc = p.semantics == GB_SEM_ACCUM_SCALAR_BETA ||
                                       (p.semantics == GB_SEM_BLAS && p.beta != 0.0);
                    for (int rb = 0; rb < rows; rb += 16) {   // sixteen rows' loads in flight at once
                        double cv[16];
                        int er[16];
#pragma unroll
                        for (int j = 0; j < 16; j++) {
                            const int rr = rb + j;
                            er[j] = rr < rows ? __ldg(p.erow + row0 + rr) : 0;
                            cv[j] = (rr < rows && needc) ? p.C[(row0 + rr) * p.ldc + col] : 0.0;
                        }
#pragma unroll
                        for (int j = 0; j < 16; j++) {
                            const int rr = rb + j;
                            if (rr >= rows) break;
                            double v;
                            if (fc == kNonFiniteLineExp || er[j] == kNonFiniteLineExp)
                                v = p.alpha * native_dot_cold(p.A, p.lda, p.ta, row0 + rr, p.B, p.ldb, p.tb, col, p.K);
                            else
                                v = p.alpha * mul_pow2(stage[rr * 33 + lane], fc);
                            if (p.semantics == GB_SEM_BLAS) {
                                if (p.beta != 0.0) v = fma(p.beta, cv[j], v);
                            } else if (p.semantics == GB_SEM_SCALAR_BETA) {
                                v = v + p.beta;
                            } else {
                                v = cv[j] + (v + p.beta);
                            }
                            p.C[(row0 + rr) * p.ldc + col] = v;
                        }
                    }
                }
                __syncwarp();
            }
            ptx::tc_fence_before();
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ------------------------------------------------------------ wide form
// 128 x 256 C tiles (BN_W = 256): every MMA is M128 N256 K16, twice the work
// of the 128 x 128 form's per instruction and per byte of V staged, and the
// W tile of a k-block serves 256 columns.  The two FP32 accumulators take all
// 512 TMEM columns, so the FP64 running sum of each diagonal flush lives in
// a per-CTA scratch array in global memory (256 KB per CTA, L2-resident,
// interleaved so that a warp's access to one pair of a lane's values is 512
// contiguous bytes).  Warps: 0 TMA, 1 MMA, 2-9 epilogue (two per TMEM lane
// quarter, 128 columns each).  The arithmetic is that of ozaki_gemm_kernel
// (same chunk sums, flush order, exact scalings and rounding), so the
// results are the same bit for bit.
namespace wide {
constexpr int BN_W = 256, STAGES_W = 4, EW = 8, NT_W = 64 + 32 * EW;
constexpr int W_TILE = BN_W * BK * 2;                       // 32 KB
constexpr int STAGE_W = TILE_BYTES + W_TILE;                // 48 KB
constexpr int SMEM_W = STAGES_W * STAGE_W + 1024 + 256;
static_assert(SMEM_W <= 232448, "shared memory");
constexpr size_t SCRATCH_DOUBLES = (size_t)EW * 32 * 128;   // per CTA
}  // namespace wide

__global__ void __launch_bounds__(wide::NT_W, 1)
    ozaki_wide_kernel(const __grid_constant__ CUtensorMap tmV, const __grid_constant__ CUtensorMap tmW, OzParams p,
                      double *scratch) {
    using namespace wide;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES_W * STAGE_W);
    uint64_t *empty = full + STAGES_W;
    uint64_t *acc_full = empty + STAGES_W;
    uint64_t *acc_empty = acc_full + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int num_tiles = p.tiles_m * p.tiles_n;
    const int nchunks = (p.num_kb + KCHUNK_BLOCKS - 1) / KCHUNK_BLOCKS;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES_W; s++) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            ptx::mbar_init(&acc_full[b], 1);
            ptx::mbar_init(&acc_empty[b], EW);
        }
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&tmV);
        ptx::tma_prefetch_desc(&tmW);
    }
    if (warp == 1) ptx::tmem_alloc(tmem_slot, TMEM_COLS);
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {   // TMA producer: per tile, per pair, every K block
            int kbg = 0;
            bool go = true;
            for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
                int tm, tn;
                tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
                for (int q = 0; q < p.npairs && go; q++) {
                    const int vrow = (int)((p.pt[q] - 1) * p.mp + (int64_t)tm * BM);
                    const int wrow = (int)((p.pu[q] - 1) * p.np + (int64_t)tn * BN_W);
                    for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
                        const int s = kbg % STAGES_W;
                        if (kbg >= STAGES_W && !ptx::mbar_wait(&empty[s], ((kbg / STAGES_W) & 1) ^ 1, p.err, 11)) {
                            go = false;
                            break;
                        }
                        uint8_t *st = smem + s * STAGE_W;
                        ptx::mbar_arrive_expect_tx(&full[s], STAGE_W);
                        ptx::tma_load_2d(st, &tmV, &full[s], kb * BK, vrow);
                        ptx::tma_load_2d(st + TILE_BYTES, &tmW, &full[s], kb * BK, wrow);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer: one accumulator per K chunk of a pair
            constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, BN_W);
            int kbg = 0, gi = 0;
            bool go = true;
            for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
                for (int q = 0; q < p.npairs && go; q++) {
                    for (int c = 0; c < nchunks && go; c++, gi++) {
                        const int b = gi & 1;
                        if (gi >= 2 && !ptx::mbar_wait(&acc_empty[b], ((gi >> 1) & 1) ^ 1, p.err, 12)) {
                            go = false;
                            break;
                        }
                        ptx::tc_fence_after();
                        const uint32_t acc = tmem + (uint32_t)(b * BN_W);
                        const int kb_end = min(p.num_kb, (c + 1) * KCHUNK_BLOCKS);
                        for (int kb = c * KCHUNK_BLOCKS; kb < kb_end; kb++, kbg++) {
                            const int s = kbg % STAGES_W;
                            if (!ptx::mbar_wait(&full[s], (kbg / STAGES_W) & 1, p.err, 13)) {
                                go = false;
                                break;
                            }
                            ptx::tc_fence_after();
                            const uint32_t st = ptx::smem_u32(smem + s * STAGE_W);
                            const uint64_t vd = ptx::sdesc_kmajor_sw128(st);
                            const uint64_t wd = ptx::sdesc_kmajor_sw128(st + TILE_BYTES);
#pragma unroll
                            for (int k = 0; k < BK / 16; k++) {
                                const uint64_t dk = (uint64_t)((k * 32) >> 4);
                                ptx::umma_f16(acc, vd + dk, wd + dk, idesc, (kb != c * KCHUNK_BLOCKS) || (k != 0));
                            }
                            ptx::umma_commit(&empty[s]);
                        }
                        if (go) ptx::umma_commit(&acc_full[b]);
                    }
                }
            }
        }
    } else {   // epilogue warps 2..9: TMEM lane quarter warp % 4, columns 128 * ((warp - 2) / 4) + 0..127
        const int w = warp - 2, q = warp % 4;
        // this lane's value pair jp at scr[jp * 32] (formed where used: registers are tight here)
#define OZ_SCR (reinterpret_cast<double2 *>(scratch + (size_t)blockIdx.x * SCRATCH_DOUBLES) + \
                (size_t)(threadIdx.x / 32 - 2) * 64 * 32 + threadIdx.x % 32)
        int gi = 0;
        bool go = true;
        for (int t = blockIdx.x; t < num_tiles && go; t += gridDim.x) {
            bool first_flush = true;
            int iacc[128];
#pragma unroll
            for (int j = 0; j < 128; j++) iacc[j] = 0;
            int nacc = 0;
            for (int qq = 0; qq < p.npairs && go; qq++) {
                const int lev = p.pt[qq] + p.pu[qq];
                const bool lev_ends = qq == p.npairs - 1 || p.pt[qq + 1] + p.pu[qq + 1] != lev;
                for (int c = 0; c < nchunks; c++, gi++) {
                    const int b = gi & 1;
                    if (!ptx::mbar_wait(&acc_full[b], (gi >> 1) & 1, p.err, 14)) { go = false; break; }
                    ptx::tc_fence_after();
#pragma unroll
                    for (int cb = 0; cb < 8; cb++) {   // 16 columns per load
                        uint32_t r[16];
                        ptx::tmem_ld_32x32b_x16(tmem + (uint32_t)(b * BN_W) + ((uint32_t)(q * 32) << 16) +
                                                    (uint32_t)((w / 4) * 128 + cb * 16), r);
                        ptx::tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 16; j++) iacc[cb * 16 + j] += __float2int_rn(__uint_as_float(r[j]));
                    }
                    ptx::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) ptx::mbar_arrive(&acc_empty[b]);
                    const bool flush = (c == nchunks - 1 && lev_ends) || ++nacc == MAX_CHUNKS_INT32;
                    if (flush) {   // FP64 sum += 2^(2-8(t+u)) * iacc (exact scaling, one rounding)
                        nacc = 0;
                        const double scale = __longlong_as_double((long long)(1023 + 2 - 8 * lev) << 52);
                        double2 *scr = OZ_SCR;
                        if (first_flush) {
#pragma unroll
                            for (int jp = 0; jp < 64; jp++)
                                scr[jp * 32] = make_double2(fma((double)iacc[2 * jp], scale, 0.0),
                                                            fma((double)iacc[2 * jp + 1], scale, 0.0));
                        } else {
#pragma unroll
                            for (int g8 = 0; g8 < 64; g8 += 4) {   // four pairs' loads in flight
                                double2 v[4];
#pragma unroll
                                for (int i = 0; i < 4; i++) v[i] = __ldcg(scr + (g8 + i) * 32);
#pragma unroll
                                for (int i = 0; i < 4; i++) {
                                    v[i].x = fma((double)iacc[2 * (g8 + i)], scale, v[i].x);
                                    v[i].y = fma((double)iacc[2 * (g8 + i) + 1], scale, v[i].y);
                                    __stcg(scr + (g8 + i) * 32, v[i]);
                                }
                            }
                        }
#pragma unroll
                        for (int j = 0; j < 128; j++) iacc[j] = 0;
                        first_flush = false;
                    }
                }
            }
            if (!go) break;
            // C = alpha * 2^(e_i + f_j) * sum (+ beta ...): this lane's row, 128 columns
            int tm, tn;
            tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
            const int64_t row = (int64_t)tm * BM + q * 32 + lane;
            const int64_t c0 = (int64_t)tn * BN_W + (w / 4) * 128;
            const bool rowok = row < p.M;
            const int erow = rowok ? p.erow[row] : 0;
            const bool needc = p.semantics == GB_SEM_ACCUM_SCALAR_BETA || (p.semantics == GB_SEM_BLAS && p.beta != 0.0);
            double *crow = p.C + row * p.ldc;
            const double2 *scr = OZ_SCR;
#pragma unroll 1
            for (int g8 = 0; g8 < 64; g8 += 4) {   // eight columns at a time, their C loads in flight together
                double2 sm[4];
                double cv[8];
#pragma unroll
                for (int i = 0; i < 4; i++) sm[i] = __ldcg(scr + (g8 + i) * 32);
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int64_t col = c0 + 2 * g8 + j;
                    cv[j] = (rowok && needc && col < p.N) ? crow[col] : 0.0;
                }
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int64_t col = c0 + 2 * g8 + j;
                    if (!rowok || col >= p.N) continue;
                    const int fc = __ldg(p.fcol + col);
                    const double sum = (j & 1) ? sm[j / 2].y : sm[j / 2].x;
                    double v;
                    if (fc == kNonFiniteLineExp || erow == kNonFiniteLineExp)
                        v = p.alpha * native_dot_cold(p.A, p.lda, p.ta, row, p.B, p.ldb, p.tb, col, p.K);
                    else
                        v = p.alpha * mul_pow2(mul_pow2(sum, erow), fc);
                    if (p.semantics == GB_SEM_BLAS) {
                        if (p.beta != 0.0) v = fma(p.beta, cv[j], v);
                    } else if (p.semantics == GB_SEM_SCALAR_BETA) {
                        v = v + p.beta;
                    } else {
                        v = cv[j] + (v + p.beta);
                    }
                    crow[col] = v;
                }
            }
        }
    }

#undef OZ_SCR
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

}  // namespace

static gb_status ozaki_one(const GemmArgs &g, int s);

// Exponents e of `lines` lines of `len` FP64 values (max |x| < 2^e, 0 for an
// all-zero line): line i at X + i*ld (contiguous) or, strided, element k of
// line i at X[k*ld + i].
gb_status ozaki_line_exponents(const double *X, int64_t ld, bool strided, int64_t lines, int64_t len, int *e,
                               cudaStream_t st) {
    if (lines <= 0) return ok();
    if (!strided) maxexp_contig_kernel<<<(unsigned)ceil_div(lines, 8), 256, 0, st>>>(X, ld, lines, len, e);
    else launch_maxexp_strided(X, ld, lines, len, e, st);
    GB_LAUNCH_CHECK("ozaki exponents");
    return ok();
}

// Slices of both operands take s * (Mp + Np) * Kp * 2 bytes of workspace.
// Past kWorkspaceCap the K range is cut into chunks, each sliced and
// multiplied on its own and accumulated into C (beta applied by the first
// chunk, later chunks add with beta = 1); each chunk gets its own row and
// column exponents.
constexpr double kWorkspaceCap = 4.0 * (1ull << 30);

gb_status launch_dgemm_ozaki(const GemmArgs &g, int slices) {
    if (g.M == 0 || g.N == 0) return ok();
    const int s = slices > 0 ? slices : ozaki_pick_slices(0.0, g.K);
    if (s < 2 || s > MAXS) return set_status(GB_ERR_INVALID_ARG, "ozaki: slices %d not in 2..%d", s, MAXS);
    const double per_k = (double)s * (double)(ceil_div(g.M, BM) * BM + ceil_div(g.N, BN) * BN) * 2.0;
    int64_t kc = (int64_t)(kWorkspaceCap / per_k) / (KCHUNK_BLOCKS * BK) * (KCHUNK_BLOCKS * BK);
    if (kc < KCHUNK_BLOCKS * BK) kc = KCHUNK_BLOCKS * BK;
    if (g.K <= kc) return ozaki_one(g, s);
    for (int64_t k0 = 0; k0 < g.K; k0 += kc) {
        GemmArgs c = g;
        c.K = (g.K - k0) < kc ? (g.K - k0) : kc;
        c.A = (const double *)g.A + (g.ta ? k0 * g.lda : k0);
        c.B = (const double *)g.B + (g.tb ? k0 : k0 * g.ldb);
        if (k0 > 0) {   // later chunks: C += alpha * A_k B_k
            c.semantics = GB_SEM_BLAS;
            c.beta = 1.0;
        }
        gb_status st = ozaki_one(c, s);
        if (st != GB_OK) return st;
    }
    return ok();
}

static gb_status ozaki_one(const GemmArgs &g, int s) {
    // the wide form (128 x 256 tiles) once op(B) has 256 columns; GB_OZAKI_WIDE=0 keeps 128 x 128
    const char *wv = getenv("GB_OZAKI_WIDE");
    const bool wide = !(wv && wv[0] == '0') && g.N >= wide::BN_W;
    const int bn = wide ? wide::BN_W : BN;
    const int64_t kp = ceil_div(g.K, BK) * BK;
    const int64_t mp = ceil_div(g.M, BM) * BM, np = ceil_div(g.N, bn) * bn;
    if (s * mp > 0x7fffffff || s * np > 0x7fffffff || kp > 0x7fffffff)
        return set_status(GB_ERR_UNSUPPORTED, "ozaki: problem too large for 32-bit TMA coordinates");
    const size_t ebytes = ((size_t)(mp + np) * sizeof(int) + 255) / 256 * 256;
    const size_t vbytes = (size_t)s * mp * kp * 2, wbytes = (size_t)s * np * kp * 2;
    const int64_t tiles_total = (mp / BM) * (np / bn);
    const int grid = (int)(tiles_total < sm_count() ? tiles_total : sm_count());
    const size_t sbytes = wide ? (size_t)grid * wide::SCRATCH_DOUBLES * sizeof(double) : 0;
    uint8_t *ws = (uint8_t *)workspace(vbytes + wbytes + ebytes + sbytes + 4096, g.stream);
    if (!ws) return (gb_status)gb_get_last_status();
    unsigned short *V = (unsigned short *)ws;
    unsigned short *W = (unsigned short *)(ws + vbytes);
    int *erow = (int *)(ws + vbytes + wbytes);
    int *fcol = erow + mp;
    double *scratch = wide ? (double *)(ws + vbytes + wbytes + ebytes) : nullptr;   // 256-byte aligned
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "ozaki: no device error word");

    // exponents: rows of op(A), columns of op(B)
    const double *A = (const double *)g.A, *B = (const double *)g.B;
    if (!g.ta) {
        maxexp_contig_kernel<<<(unsigned)ceil_div(g.M, 8), 256, 0, g.stream>>>(A, g.lda, g.M, g.K, erow);
    } else {
        launch_maxexp_strided(A, g.lda, g.M, g.K, erow, g.stream);
    }
    GB_LAUNCH_CHECK("ozaki exponents A");
    if (g.tb) {
        maxexp_contig_kernel<<<(unsigned)ceil_div(g.N, 8), 256, 0, g.stream>>>(B, g.ldb, g.N, g.K, fcol);
    } else {
        launch_maxexp_strided(B, g.ldb, g.N, g.K, fcol, g.stream);
    }
    GB_LAUNCH_CHECK("ozaki exponents B");

    // digits: V_t = digits of op(A) rows (M x K), W_u = digits of op(B)^T rows (N x K)
    dim3 gA((unsigned)ceil_div(kp, 32), (unsigned)ceil_div(mp, 32));
    dim3 gB((unsigned)ceil_div(kp, 32), (unsigned)ceil_div(np, 32));
    if (gA.y > 65535u || gB.y > 65535u) return set_status(GB_ERR_UNSUPPORTED, "ozaki: M or N too large");
    slice_kernel<<<gA, 256, 0, g.stream>>>(A, g.lda, g.ta ? 1 : 0, g.M, g.K, mp, kp, erow, s, V);
    GB_LAUNCH_CHECK("ozaki slices A");
    slice_kernel<<<gB, 256, 0, g.stream>>>(B, g.ldb, g.tb ? 0 : 1, g.N, g.K, np, kp, fcol, s, W);
    GB_LAUNCH_CHECK("ozaki slices B");

    CUtensorMap tV, tW;
    if (!make_tmap_bf16(&tV, V, kp, (uint64_t)s * mp, kp * 2, BK, BM, 128) ||
        !make_tmap_bf16(&tW, W, kp, (uint64_t)s * np, kp * 2, BK, bn, 128))
        return set_status(GB_ERR_CUDA, "ozaki: cuTensorMapEncodeTiled failed");

    OzParams p{};
    p.C = (double *)g.C; p.M = g.M; p.N = g.N; p.ldc = g.ldc;
    p.alpha = g.alpha; p.beta = g.beta; p.semantics = g.semantics;
    p.num_kb = (int)(kp / BK);
    p.tiles_m = (int)(mp / BM); p.tiles_n = (int)(np / bn);
    p.mp = mp; p.np = np;
    p.erow = erow; p.fcol = fcol; p.err = err;
    p.A = A; p.B = B; p.lda = g.lda; p.ldb = g.ldb; p.K = g.K; p.ta = g.ta ? 1 : 0; p.tb = g.tb ? 1 : 0;
    // slice pairs t + u <= s + 1, diagonal by diagonal, least significant
    // first: the pairs of a diagonal share a scale, so the epilogue sums them
    // exactly in int32 and flushes to FP64 once per diagonal (GB300's FP64
    // pipe made one flush per pair the limiter).  GB_OZAKI_PAIR_ORDER=w
    // groups the pairs by the W digit u instead: the tiles in flight (8 tile
    // rows x 19 tile columns) keep W_u's panels hot in L2, halving the DRAM
    // reads, at one flush per pair.
    const char *ord = getenv("GB_OZAKI_PAIR_ORDER");
    int n = 0;
    if (!(ord && ord[0] == 'w')) {
        for (int d = s + 1; d >= 2; d--)
            for (int t = 1; t <= s; t++) {
                int u = d - t;
                if (u >= 1 && u <= s) { p.pt[n] = (signed char)t; p.pu[n] = (signed char)u; n++; }
            }
    } else {
        for (int u = s; u >= 1; u--)
            for (int t = s + 1 - u; t >= 1; t--) { p.pt[n] = (signed char)t; p.pu[n] = (signed char)u; n++; }
    }
    p.npairs = n;

    static std::atomic<uint64_t> attr{0};
    if (device_setup_needed(attr)) {
        GB_CUDA_TRY(cudaFuncSetAttribute(ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        GB_CUDA_TRY(cudaFuncSetAttribute(ozaki_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, wide::SMEM_W));
        device_setup_done(attr);
    }
    if (wide) {
        ozaki_wide_kernel<<<grid, wide::NT_W, wide::SMEM_W, g.stream>>>(tV, tW, p, scratch);
        GB_LAUNCH_CHECK("ozaki_wide_kernel");
    } else {
        ozaki_gemm_kernel<<<grid, NT, SMEM_BYTES, g.stream>>>(tV, tW, p);
        GB_LAUNCH_CHECK("ozaki_gemm_kernel");
    }
    return ok();
}

}  // namespace gb
