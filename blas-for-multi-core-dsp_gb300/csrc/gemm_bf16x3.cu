// gemm_bf16x3.cu -- SGEMM as sums of 16-bit piece products on the tcgen05
// tensor cores, FP32 accumulation.
//
// C = alpha * op(A) op(B) (+ beta C / + beta), FP32 in and out.  Each FP32
// operand value is cut into 16-bit pieces and the piece products that carry
// FP32's precision are accumulated in FP32 in tensor memory.  These are the
// precision forms of the reference's FP32 SGEMM (sgemm_release_V1.3.2/
// device_code/sgemm_kernel.c:2476-4505); none has a counterpart there.
//  - BF16X3: x_hi = bf16(x), x_lo = bf16(x - x_hi); a_hi*b_hi + a_hi*b_lo +
//    a_lo*b_hi (the a_lo*b_lo term, ~2^-16 relative, is dropped; hi + lo
//    carry ~16 of FP32's 24 bits).
//  - BF16X6: three BF16 pieces (24 bits), the six products of weight >=
//    2^-16, the accumulator restarted every 256 k and folded in registers.
//  - FP16X3: every row of op(A) and column of op(B) scaled by a power of two
//    that puts its largest magnitude in [2^14, 2^15), then x_hi = fp16(x),
//    x_lo = fp16(x - x_hi) (22 bits), the same three products as BF16X3, the
//    accumulator restarted every 128 k and folded in registers, and the
//    scales undone exactly in the epilogue.
//
// Kernels:
//  1. (FP16X3) scan: the largest |x| of every row of op(A) and column of op(B).
//  2. split: op(A) -> pieces (M x Kp, K-major), op(B) -> pieces (N x Kp,
//     K-major), Kp = K rounded up to 64 with zeros.  The transpose modes are
//     absorbed here (a row-major or a transposed read, always a K-major
//     write), so the GEMM kernel has one operand layout.
//  3. gemm: persistent, one CTA per SM over 128 x 256 C tiles, K in blocks of
//     32 (one 64-byte swizzle atom), a 4-stage TMA -> shared memory pipeline
//     with mbarriers; warp 0 issues TMA, warp 1 issues tcgen05.mma (M=128,
//     N=256, K=16, three products per K step into a TMEM accumulator of 256
//     columns, two accumulators alternating), the epilogue warps read the
//     finished accumulator with tcgen05.ld and write C with alpha/beta.
// Skinny products (min(M, N) <= 64) run BF16X3 in one fused kernel instead
// (TMA of the FP32 tiles, converter warps, MMA).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

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

// ------------------------------------------------------------ FP16 scaling
// The FP16 form (FP16X3) carries each FP32 value as two FP16 pieces, 11 + 11
// significand bits, after scaling its line -- a row of op(A) or a column of
// op(B) -- by a power of two that puts the line's largest magnitude in
// [2^14, 2^15): FP16 cannot overflow there, and what falls below FP16's
// subnormal floor (2^-24) is 2^-38 of the line's maximum or less.  The
// epilogue undoes both scalings exactly.  (Three-product FP16 splitting
// with scaling is the method of Ootomo & Yokota, "Recovering single
// precision accuracy from Tensor Cores while surpassing the FP32 theoretical
// peak performance", IJHPCA 2022; the per-line power-of-two scaling and the
// folded accumulation here are this library's.)

// Scale exponent s of a line from the bit pattern of its largest |x|:
// max * 2^s in [2^14, 2^15).  0 for an all-zero line; kNonFiniteScale for a
// line holding an Inf or a NaN (whose outputs the epilogue recomputes as
// plain dot products).
constexpr int kNonFiniteScale = -100000;
__device__ __forceinline__ int f16_line_scale(unsigned mb) {
    if (mb == 0u) return 0;
    if (mb >= 0x7f800000u) return kNonFiniteScale;
    const int e = mb >= 0x00800000u ? (int)(mb >> 23) - 127 : (31 - __clz((int)mb)) - 149;
    return 14 - e;   // -113 .. 163
}

__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }   // -126 <= k <= 127

// x * 2^s for s in [-113, 163]: exact, in two steps above 2^127 (the line's
// maximum is then below 2^-113, so the first step cannot overflow)
__device__ __forceinline__ float scale_line(float x, int s) {
    return s > 127 ? (x * pow2f(127)) * pow2f(s - 127) : x * pow2f(s);
}

// x * 2^k, branch-free, as two factors in the normal range applied largest
// first: exact while the result is normal, and for k in [-252, 254] the
// product of the factors is 2^k; the epilogue's k lies in [-326, 226] and
// below -252 the result underflows to zero either way (|x| < 2^62).
__device__ __forceinline__ float mul_pow2f(float x, int k) {
    const int a = max(-126, min(127, k));
    const int b = max(-126, min(127, k - a));
    return x * pow2f(a) * pow2f(b);
}

// Plain FP32 dot product of row i of op(A) and column j of op(B), in k order:
// the outputs whose line holds an Inf or a NaN, so that those propagate as
// IEEE arithmetic has them.
__device__ __forceinline__ float dot_f32_cold(const float *A, int64_t lda, int ta, int64_t i, const float *B,
                                              int64_t ldb, int tb, int64_t j, int64_t K) {
    float s = 0.f;
    for (int64_t k = 0; k < K; k++) {
        const float a = ta ? A[k * lda + i] : A[i * lda + k];
        const float b = tb ? B[j * ldb + k] : B[k * ldb + j];
        s = fmaf(a, b, s);
    }
    return s;
}

// ------------------------------------------------------ programmatic launch
// A split pass may be launched (programmatic stream serialization) to run
// beside the previous call's GEMM on the same stream, which triggers its
// dependents as it starts.  The host allows that only when this call's A and
// B do not overlap the previous GEMM's C.  What the host cannot see is work
// the caller queued between the two calls: with such work in between, the
// split starts only once that work has finished (it does not trigger early),
// and by then the previous GEMM has finished as well.  So each CTA reads the
// count of finished GEMM CTAs: below `expect` (the CTAs launched up to and
// including the previous GEMM), the previous GEMM is still running and is the
// split's immediate predecessor, and A and B are safe to read; otherwise it
// waits for the preceding grid's completion and memory flush before reading.
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void split_entry_guard(const unsigned long long *done, unsigned long long expect) {
    __shared__ int must_wait;
    if (threadIdx.x == 0) must_wait = done == nullptr || ld_acquire_u64(done) >= expect;
    __syncthreads();
    if (must_wait) ptx::pdl_wait();   // returns at once when not launched as a dependent
}

// ------------------------------------------------------------------ scan
// Largest |x| bit pattern of every row of op(X) (rows x K) -- non-negative
// floats order as their bit patterns -- by atomicMax from 64 x 256 tiles.
// Each line's entry is (gen << 32) | bits with the call's generation `gen`
// (larger than any earlier call's on the stream), so no clearing is needed
// between calls: every line receives its call's value, which is larger than
// whatever an earlier call left.  Both operands in one launch; `vec`: 16-byte
// loads.  The scan may be launched beside the previous call's GEMM, like a
// split pass (split_entry_guard); each CTA then counts itself in `scan_done`
// and triggers the split pass that follows, which waits for the count
// instead of the scan's completion, so both can run beside that GEMM.
struct ScanOp {
    const float *X;
    int64_t ldx, rows, tiles_k, tiles;
    int trans;                      // element (r, k) at X[k*ldx + r]
    unsigned long long *out;
};
struct ScanArgs {
    ScanOp op[2];
    int64_t K;
    int vec;
    unsigned gen;
    const unsigned long long *done;   // split_entry_guard
    unsigned long long expect;
    unsigned long long *scan_done;    // finished scan CTAs of the stream (null: not counted)
};

__device__ __forceinline__ unsigned absbits(float x) { return __float_as_uint(x) & 0x7fffffffu; }

__global__ void __launch_bounds__(256) maxbits_kernel(const __grid_constant__ ScanArgs a) {
    __shared__ unsigned red[16][65];
    split_entry_guard(a.done, a.expect);
    int64_t b = blockIdx.x;
    const int w = b < a.op[0].tiles ? 0 : 1;
    if (w) b -= a.op[0].tiles;
    const ScanOp &o = a.op[w];
    // a CTA: 64 lines x 256 k (four 64-k blocks), one atomic per line
    const int64_t r0 = (b / o.tiles_k) * 64, kb0 = (b % o.tiles_k) * 256;
    const int t = threadIdx.x, c4 = 4 * (t % 16), rl = t / 16;
    const unsigned long long tag = (unsigned long long)a.gen << 32;
    if (!o.trans) {   // 16 threads (a half warp) per row, 4 k each
        unsigned m[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int sb = 0; sb < 4; sb++) {
            const int64_t k = kb0 + 64 * sb + c4;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int64_t r = r0 + rl + 16 * i;
                if (r >= o.rows || k >= a.K) continue;
                const float *src = o.X + r * o.ldx + k;
                if (a.vec && k + 3 < a.K) {
                    const float4 x = __ldg(reinterpret_cast<const float4 *>(src));
                    m[i] = max(m[i], max(max(absbits(x.x), absbits(x.y)), max(absbits(x.z), absbits(x.w))));
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (k + q < a.K) m[i] = max(m[i], absbits(src[q]));
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int64_t r = r0 + rl + 16 * i;
            unsigned mi = m[i];
#pragma unroll
            for (int s = 8; s >= 1; s >>= 1) mi = max(mi, __shfl_xor_sync(0xffffffffu, mi, s));
            if ((t & 15) == 0 && r < o.rows) atomicMax(&o.out[r], tag | mi);
        }
    } else {
        unsigned m[4] = {0u, 0u, 0u, 0u};   // 4 consecutive rows, 4 k each per 64-k block
#pragma unroll
        for (int sb = 0; sb < 4; sb++) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int64_t k = kb0 + 64 * sb + rl + 16 * i, r = r0 + c4;
                if (k >= a.K) continue;
                const float *src = o.X + k * o.ldx + r;
                if (a.vec && r + 3 < o.rows) {
                    const float4 x = __ldg(reinterpret_cast<const float4 *>(src));
                    m[0] = max(m[0], absbits(x.x)); m[1] = max(m[1], absbits(x.y));
                    m[2] = max(m[2], absbits(x.z)); m[3] = max(m[3], absbits(x.w));
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (r + q < o.rows) m[q] = max(m[q], absbits(src[q]));
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) red[rl][c4 + q] = m[q];
        __syncthreads();
        if (t < 64) {
            unsigned mm = 0;
#pragma unroll
            for (int j = 0; j < 16; j++) mm = max(mm, red[j][t]);
            if (r0 + t < o.rows) atomicMax(&o.out[r0 + t], tag | mm);
        }
    }
    // this CTA's maxima are in: count it, then let the split pass launch
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        if (a.scan_done) atomicAdd(a.scan_done, 1ull);
        ptx::pdl_launch_dependents();
    }
    // as split_kernel: the grid does not complete before the previous grid has
    if (blockIdx.x == 0 && threadIdx.x == 0) ptx::pdl_wait();
}

// The split pass of the FP16 form waits for every CTA of its scan: `expect`
// finished scan CTAs on the stream (bounded; on expiry the error word is set
// and the pass goes on, so nothing hangs).
__device__ __forceinline__ void scan_entry_wait(const unsigned long long *scan_done, unsigned long long expect,
                                                int *err) {
    if (threadIdx.x == 0 && ld_acquire_u64(scan_done) < expect) {
        const uint64_t t0 = ptx::globaltimer();
        while (ld_acquire_u64(scan_done) < expect) {
            if (ptx::globaltimer() - t0 > ptx::kWaitLimitNs) {
                atomicCAS(err, 0, 20);
                break;
            }
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------------ split
// Pieces of one value.  BF16 (F16 = false): x = hi + lo (+ lo2) exactly up
// to the last piece, each piece the rounded remainder.  FP16 (F16 = true):
// x is first scaled by its line's 2^s (s = kNonFiniteScale: the line holds
// an Inf or a NaN, its outputs are recomputed, and hi = x, lo = 0).
template <bool F16>
struct Pieces;

template <>
struct Pieces<false> {
    using T = __nv_bfloat16;
    static __device__ __forceinline__ void cut(float x, int, T &h, T &l, T &l2) {
        h = __float2bfloat16_rn(x);
        const float rem = x - __bfloat162float(h);   // exact
        l = __float2bfloat16_rn(rem);
        l2 = __float2bfloat16_rn(rem - __bfloat162float(l));
    }
    static __device__ __forceinline__ uint16_t bits(T v) { return __bfloat16_as_ushort(v); }
};

template <>
struct Pieces<true> {
    using T = __half;
    static __device__ __forceinline__ void cut(float x, int s, T &h, T &l, T &l2) {
        l2 = __float2half_rn(0.f);
        if (s == kNonFiniteScale) {
            h = __float2half_rn(x);
            l = l2;
            return;
        }
        const float v = scale_line(x, s);           // |v| < 2^15
        h = __float2half_rn(v);
        l = __float2half_rn(v - __half2float(h));   // the remainder is exact in FP32
    }
    static __device__ __forceinline__ uint16_t bits(T v) { return __half_as_ushort(v); }
};

// out_hi/out_lo(/out_lo2): rows x kp (K-major).  Source element (r, k):
// trans ? X[k*ldx + r] : X[r*ldx + k].  32x32 tiles through shared memory
// so both the read and the write are coalesced in either layout.  With
// out_lo2 the value is cut in three BF16 pieces (hi, mid, lo: 24 bits).
// mbits (FP16 form): the largest |x| bit pattern of each row (low 32 bits).
template <bool F16>
__global__ void __launch_bounds__(256) split_kernel(const float *__restrict__ X, int64_t ldx, int trans, int64_t rows,
                                                    int64_t K, int64_t kp, uint16_t *__restrict__ out_hi,
                                                    uint16_t *__restrict__ out_lo, uint16_t *__restrict__ out_lo2,
                                                    const unsigned long long *__restrict__ mbits,
                                                    const unsigned long long *done, unsigned long long expect,
                                                    const unsigned long long *scan_done,
                                                    unsigned long long scan_expect, int *err) {
    using P = Pieces<F16>;
    __shared__ float tile[32][33];
    if (scan_done) scan_entry_wait(scan_done, scan_expect, err);
    else split_entry_guard(done, expect);
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
            typename P::T h, l, l2;
            P::cut(tile[tx][ty + i], F16 ? f16_line_scale((unsigned)mbits[r]) : 0, h, l, l2);
            out_hi[r * kp + k] = P::bits(h);
            out_lo[r * kp + k] = P::bits(l);
            if (out_lo2) out_lo2[r * kp + k] = P::bits(l2);
        }
    }
    // possibly launched to overlap the previous call's GEMM: one thread keeps the grid from
    // completing before that grid has, so the stream order of the GEMM that follows is unchanged
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) ptx::pdl_wait();
}

// Vectorised split of both operands in one launch (16-byte aligned sources
// with leading dimensions a multiple of 4).  A CTA converts a 64 x 64 block
// of (row, k): a K-contiguous source is read and written 4 values at a time
// straight from registers; a row-contiguous source is read 4 rows at a time
// into shared memory and written 4 k at a time, in two halves of 32 k (a
// small tile, so that a split CTA fits on an SM beside a GEMM CTA).  Same values as
// split_kernel, about two-thirds of its time at the 4096^2 operands.
struct SplitOp {
    const float *X;
    int64_t ldx, rows, tiles_k, tiles;
    int trans;                      // source element (r, k) at X[k*ldx + r]
    uint16_t *out[3];
    const unsigned long long *mbits;   // FP16 form: largest |x| bit pattern per row (low 32 bits)
};
struct SplitArgs {
    SplitOp op[2];
    int64_t K, kp;
    int np;
    const unsigned long long *done;
    unsigned long long expect;
    const unsigned long long *scan_done;   // FP16 form: wait for the scan's CTAs (scan_entry_wait)
    unsigned long long scan_expect;
    int *err;
};

template <bool F16>
__device__ __forceinline__ void split_store4(const SplitArgs &a, const SplitOp &o, int64_t r, int64_t k,
                                             const float (&v)[4]) {
    using P = Pieces<F16>;
    const int s = F16 ? f16_line_scale((unsigned)o.mbits[r]) : 0;
    uint32_t h[2], l[2], l2[2];
#pragma unroll
    for (int q = 0; q < 4; q += 2) {
        typename P::T h0, l0, m0, h1, l1, m1;
        P::cut(v[q], s, h0, l0, m0);
        P::cut(v[q + 1], s, h1, l1, m1);
        h[q / 2] = (uint32_t)P::bits(h0) | ((uint32_t)P::bits(h1) << 16);
        l[q / 2] = (uint32_t)P::bits(l0) | ((uint32_t)P::bits(l1) << 16);
        l2[q / 2] = (uint32_t)P::bits(m0) | ((uint32_t)P::bits(m1) << 16);
    }
    const int64_t off = r * a.kp + k;
    *reinterpret_cast<uint2 *>(o.out[0] + off) = make_uint2(h[0], h[1]);
    *reinterpret_cast<uint2 *>(o.out[1] + off) = make_uint2(l[0], l[1]);
    if (a.np == 3) *reinterpret_cast<uint2 *>(o.out[2] + off) = make_uint2(l2[0], l2[1]);
}

template <bool F16>
__global__ void __launch_bounds__(256) split_vec_kernel(const __grid_constant__ SplitArgs a) {
    __shared__ float tile[32][65];   // 8.3 KB: fits beside a GEMM CTA on its SM
    if (a.scan_done) scan_entry_wait(a.scan_done, a.scan_expect, a.err);
    else split_entry_guard(a.done, a.expect);
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
            split_store4<F16>(a, o, r, k, v);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) ptx::pdl_wait();   // as split_kernel
        return;
    }
    // row-contiguous source: the 64 x 64 block in two halves of 32 k through tile[k][r]
    const int kw = 4 * (t % 8), rw = t / 8;   // writer: 4 consecutive k of row rw (+ 32)
#pragma unroll
    for (int h = 0; h < 2; h++) {
        if (h) __syncthreads();   // the first half's reads of the tile are done
#pragma unroll
        for (int i = 0; i < 2; i++) {   // tile[k][r], 4 consecutive r per load
            const int kl = rl + 16 * i;
            const int64_t k = k0 + 32 * h + kl, r = r0 + c4;
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
        for (int i = 0; i < 2; i++) {
            const int rr = rw + 32 * i;
            const int64_t r = r0 + rr;
            if (r >= o.rows) continue;
            const float v[4] = {tile[kw][rr], tile[kw + 1][rr], tile[kw + 2][rr], tile[kw + 3][rr]};
            split_store4<F16>(a, o, r, k0 + 32 * h + kw, v);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ptx::pdl_wait();   // as split_kernel
}

// ------------------------------------------------------------------- gemm
// Persistent: one CTA per SM walks the 128 x BN C tiles in a grouped order
// (GROUP_M tile rows at a time, so neighbouring CTAs share A and B tiles in
// L2).  K in blocks of 32 (one 64-byte swizzle atom), 4 shared-memory stages
// holding NP 16-bit pieces of the A and B tiles (NP = 2: hi, lo with BN =
// 256; NP = 3: hi, mid, lo with BN = 128).  Two TMEM accumulators: the
// epilogue of tile (or accumulator chunk) i overlaps the MMAs of i+1.
constexpr int BM = 128, BK = 32, STAGES = 4, GROUP_M = 8;
constexpr int A_TILE = BM * BK * 2;            // 8 KB
constexpr int EPI_BYTES = 4 * 32 * 33 * 4;     // four warps' 32 x 32 staging, padded

// EW epilogue warps: 4 (one per TMEM lane quarter, all BN columns) or 8 (two
// per lane quarter, 128 columns each: the wide folding form); both stage C
// through shared memory so that loads and stores of C are coalesced.
template <int NP, int BN, int EW>
struct TwoPass {
    static constexpr int B_TILE = BN * BK * 2;
    static constexpr int STAGE_BYTES = NP * A_TILE + NP * B_TILE;
    static constexpr int NT = 64 + 32 * EW;
    // C staging: 4 warps x 32 x 32 (padded 33), or 8 warps x 32 x 16 (padded 17)
    static constexpr int EPI = EW == 4 ? EPI_BYTES : 8 * 32 * 17 * 4;
    static constexpr int SCALES = EW == 8 ? 8 * (128 + 32) * 4 : 0;   // FP16 column and row scales per warp
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EPI + 1024 /*align*/ + 256 /*barriers*/ + SCALES;
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
    // Half-tile tail: tiles [half_start, tiles) (a last wave at most half
    // full) run as two 128-column halves on different CTAs, so the wave takes
    // half a tile time.
    int half_start;
    // CTAs of this stream's GEMMs that have finished (read by the next call's
    // split pass, see split_entry_guard); null when not tracked
    unsigned long long *done;
    // FP16 form: largest |x| bit patterns of op(A)'s rows and op(B)'s columns
    // (the scale of each line), and the operands, for the outputs recomputed
    // as plain dot products
    const unsigned long long *rowbits, *colbits;   // low 32 bits (scan entries)
    const float *A, *B;
    int64_t lda, ldb, K;
    int ta, tb;
};

// Work item i of this CTA: a whole tile (half = -1) or the left / right 128
// columns of a tail tile (half 0 / 1).
__device__ __forceinline__ bool next_item(const EpiParams &p, int num_tiles, int &i, int &tile, int &half) {
    const int t = blockIdx.x + i * gridDim.x;
    i++;
    half = -1;
    if (t < p.half_start) {
        tile = t;
        return true;
    }
    const int h = t - p.half_start;
    if (h >= 2 * (num_tiles - p.half_start)) return false;
    tile = p.half_start + h / 2;
    half = h & 1;
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

// Instruction descriptor of kind::f16 with FP16 (F16) or BF16 operands, FP32 accumulation.
template <bool F16>
__host__ __device__ constexpr uint32_t idesc_f32acc(int M, int N) {
    return F16 ? (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24) : ptx::idesc_bf16_f32(M, N);
}

__device__ __forceinline__ bool reads_c(const EpiParams &p) {
    return p.semantics == GB_SEM_ACCUM_SCALAR_BETA || (p.semantics == GB_SEM_BLAS && p.beta != 0.f);
}

// alpha/beta epilogue of one output from its product x (and C's old value
// when reads_c): C = alpha x + beta C (BLAS), alpha x + beta, C + (alpha x + beta)
// 16-byte global load / store as ordered asm: the compiler keeps a load issued ahead of the
// stores that follow it in the program (the wide form's C loads run one group ahead)
__device__ __forceinline__ float4 ldg_v4(const float *a) {
    float4 v;
    asm volatile("ld.global.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(a));
    return v;
}

__device__ __forceinline__ void stg_v4(float *a, float4 v) {
    asm volatile("st.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

__device__ __forceinline__ float epi_value(const EpiParams &p, float x, float cin) {
    const float v = p.alpha * x;
    if (p.semantics == GB_SEM_BLAS) return p.beta != 0.f ? fmaf(p.beta, cin, v) : v + 0.f;
    if (p.semantics == GB_SEM_SCALAR_BETA) return v + p.beta;
    return cin + (v + p.beta);
}

// The output (row, col) from a plain FP32 dot product (its row of op(A) or
// column of op(B) holds an Inf or a NaN), written with the epilogue.
__device__ __forceinline__ void store_recomputed(const EpiParams &p, int64_t row, int64_t col) {
    const float x = dot_f32_cold(p.A, p.lda, p.ta, row, p.B, p.ldb, p.tb, col, p.K);
    float *c = p.C + row * p.ldc + col;
    *c = epi_value(p, x, reads_c(p) ? *c : 0.f);
}

// FOLD: the tensor cores add each MMA into the FP32 accumulator with an
// error of about one unit in the last place of the accumulator, biased like
// a truncation, so over a long K the error grows with the number of MMAs and
// with the size of the running sum.  With FOLD the accumulator is restarted
// every chunk_kb k-blocks (chunk_kb * 32 values of K) and the epilogue warps
// add each chunk into an FP32 running total held in registers
// (round-to-nearest).  Two forms:
//  - BN = 128, 4 epilogue warps (BF16X6): the most significant product hi*hi
//    is accumulated apart from the cross products, so only the hi*hi MMAs add
//    into a large accumulator; TMEM: two chunk buffers of 256 columns (hi*hi
//    at +0, the rest at +128).
//  - BN = 256, 8 epilogue warps (FP16X3, BF16X3 folded): all products in one
//    accumulator of 256 columns, two chunk buffers; each epilogue warp keeps
//    the totals of 32 rows x 128 columns and writes C through shared memory
//    16 columns at a time.
// The MMAs of chunk c+1 overlap the fold of chunk c.
// F16: FP16 pieces of scaled lines (FP16X3), the epilogue applies the scales.
template <int NP, int BN, bool FOLD, bool F16, int EW>
__global__ void __launch_bounds__(64 + 32 * EW, 1)
    bf16x3_gemm_kernel(const __grid_constant__ PieceMaps maps, EpiParams p) {
    // the next call's split pass may start beside this grid (it writes the other workspace half)
    if (threadIdx.x == 0) ptx::pdl_launch_dependents();
    using CF = TwoPass<NP, BN, EW>;
    constexpr bool SEP = FOLD && EW == 4;   // hi*hi apart from the cross products
    static_assert(!SEP || BN == 128, "the separated folding form keeps a 128-column total per thread");
    static_assert(EW == 4 || (FOLD && BN == 256), "eight epilogue warps: the wide folding form");
    static_assert(!F16 || EW == 8, "FP16 pieces: the wide folding form");
    constexpr int B_TILE = CF::B_TILE, STAGE_BYTES = CF::STAGE_BYTES;
    constexpr uint32_t ACC_COLS = SEP ? 256 : BN, TMEM_COLS = 2 * ACC_COLS;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    float *epi = reinterpret_cast<float *>(smem + STAGES * STAGE_BYTES);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES + CF::EPI);
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;     // [2]
    uint64_t *acc_empty = acc_full + 2;      // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);
    int *col_scale = reinterpret_cast<int *>(smem + STAGES * STAGE_BYTES + CF::EPI + 256);   // [8][128]
    int *row_scale = col_scale + 8 * 128;                                                     // [8][32]

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
            ptx::mbar_init(&acc_empty[b], EW);   // one arrive per epilogue warp
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
            int it = 0, t, half;
            while (go && next_item(p, num_tiles, it, t, half)) {
                int tm, tn;
                tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
                const int m0 = tm * BM, n0 = tn * BN + (half > 0 ? BN / 2 : 0);
                const uint32_t bytes = half < 0 ? STAGE_BYTES : NP * A_TILE + NP * (B_TILE / 2);
                for (int kb = 0; kb < p.num_kb; kb++, kbg++) {
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
            constexpr uint32_t idesc = idesc_f32acc<F16>(BM, BN);
            constexpr uint32_t idesc_half = idesc_f32acc<F16>(BM, BN / 2);
            int kbg = 0, ch = 0;   // running k-block and accumulator-chunk counters
            bool go = true;
            int it = 0, t, half;
            while (go && next_item(p, num_tiles, it, t, half)) {
                const uint32_t id = half < 0 ? idesc : idesc_half;
                const int nch = (p.num_kb + chunk_kb - 1) / chunk_kb;
                for (int c = 0; c < nch && go; c++, ch++) {
                    const int b = ch & 1;
                    if (ch >= 2 && !ptx::mbar_wait(&acc_empty[b], ((ch >> 1) & 1) ^ 1, p.err, 2)) {
                        go = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const uint32_t acc = tmem + (uint32_t)(b * ACC_COLS);
                    const uint32_t acc_lo = SEP ? acc + 128u : acc;   // cross products
                    const int kbc = c * chunk_kb;
                    const int kb1 = kbc + chunk_kb < p.num_kb ? kbc + chunk_kb : p.num_kb;
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
                            // advance 16 values = 32 bytes along K inside the 64-byte swizzle atom
                            const uint64_t dk = (uint64_t)((k * 32) >> 4);
                            // piece products (i, j) with i + j < NP, least significant first
#pragma unroll
                            for (int d = NP - 1; d >= 0; d--)
#pragma unroll
                                for (int i = d; i >= 0; i--) {
                                    const bool lead = SEP ? (d == NP - 1 && i == d) || d == 0 : d == NP - 1 && i == d;
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
    } else if constexpr (EW == 4) {   // epilogue: warps 2..5 own TMEM lane quarters (warp % 4)
        const int q = warp % 4;
        float *stage = epi + q * 32 * 33;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int ch = 0;
        float total[FOLD ? BN : 1];
        bool go = true;
        int it = 0, t, half;
        while (go && next_item(p, num_tiles, it, t, half)) {
            int tm, tn;
            tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
            const int64_t row0 = (int64_t)tm * BM + q * 32;
            const int64_t n0 = (int64_t)tn * BN + (half > 0 ? BN / 2 : 0);
            const int ncols = half < 0 ? BN : BN / 2;
            uint32_t accb = 0;
            if (FOLD) {
#pragma unroll
                for (int j = 0; j < (FOLD ? BN : 1); j++) total[j] = 0.f;
                for (int c = 0; c < (p.num_kb + chunk_kb - 1) / chunk_kb; c++, ch++) {
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
                const int64_t col = n0 + c + lane;
                if (col < p.N) {
                    const int rows = (p.M - row0) < 32 ? (int)(p.M - row0) : 32;
                    if (!reads_c(p)) {
                        const float add = p.semantics == GB_SEM_SCALAR_BETA ? p.beta : 0.f;
                        for (int rr = 0; rr < rows; rr++)
                            p.C[(row0 + rr) * p.ldc + col] = p.alpha * stage[rr * 33 + lane] + add;
                    } else {
                        float cin[32];
#pragma unroll
                        for (int rr = 0; rr < 32; rr++)
                            cin[rr] = rr < rows ? p.C[(row0 + rr) * p.ldc + col] : 0.f;
#pragma unroll
                        for (int rr = 0; rr < 32; rr++)
                            if (rr < rows) p.C[(row0 + rr) * p.ldc + col] = epi_value(p, stage[rr * 33 + lane], cin[rr]);
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
        }
    } else {   // EW == 8: two warps per TMEM lane quarter, 128 columns each
        // Registers: the 128 running totals and 16 columns in flight leave ~24 of the 168 for
        // everything else, so only the tile index and chunk counter stay live across the fold;
        // coordinates and pointers are recomputed after it.
        int ch = 0;
        float total[128];
        bool go = true;
        int it = 0, t, half;
        while (go && next_item(p, num_tiles, it, t, half)) {
            if (F16) {   // the scales of the warp's rows and columns, once per tile
                int tm, tn;
                tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
                const int64_t row0 = (int64_t)tm * BM + (warp % 4) * 32;
                const int64_t c0 = (int64_t)tn * BN + (half < 0 ? ((warp - 2) / 4) * 128 : half * 128);
                unsigned cb[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int64_t col = c0 + lane + 32 * j;
                    cb[j] = col < p.N ? (unsigned)p.colbits[col] : 0u;
                }
                const unsigned rb = row0 + lane < p.M ? (unsigned)p.rowbits[row0 + lane] : 0u;
                int *cs_w = col_scale + (warp - 2) * 128;
                __syncwarp();   // the previous tile's reads of the scales are done
#pragma unroll
                for (int j = 0; j < 4; j++) cs_w[lane + 32 * j] = f16_line_scale(cb[j]);
                row_scale[(warp - 2) * 32 + lane] = f16_line_scale(rb);
                __syncwarp();
            }
#pragma unroll
            for (int j = 0; j < 128; j++) total[j] = 0.f;
            const int nch = (p.num_kb + chunk_kb - 1) / chunk_kb;
            for (int c = 0; c < nch; c++, ch++) {
                const int b = ch & 1;
                if (!ptx::mbar_wait(&acc_full[b], (ch >> 1) & 1, p.err, 4)) { go = false; break; }
                ptx::tc_fence_after();
                const uint32_t a0 = tmem + (uint32_t)(b * ACC_COLS) + ((uint32_t)((warp % 4) * 32) << 16) +
                                    (uint32_t)(((warp - 2) / 4) * 128);
#pragma unroll
                for (int g = 0; g < 8; g++) {   // 16 columns per load
                    uint32_t r[16];
                    ptx::tmem_ld_32x32b_x16(a0 + (uint32_t)(g * 16), r);
                    ptx::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 16; j++) total[g * 16 + j] += __uint_as_float(r[j]);
                }
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&acc_empty[b]);
            }
            if (!go) break;
            // a half tile of the tail (128 columns in accumulator columns 0..127) is stored by the
            // warps of column half 0; the other four folded columns the MMA did not write
            const int tl = blockIdx.x + (it - 1) * gridDim.x;
            const int hf = tl < p.half_start ? -1 : ((tl - p.half_start) & 1);
            if (hf >= 0 && warp >= 6) continue;
            int tm, tn;
            tile_coords(t, p.tiles_m, p.tiles_n, tm, tn);
            const int wi = warp - 2;
            const int64_t row0 = (int64_t)tm * BM + (warp % 4) * 32;
            const int64_t c0 = (int64_t)tn * BN + (hf < 0 ? (wi / 4) * 128 : hf * 128);
            const int *cs_w = col_scale + wi * 128;
            const int *rs_w = row_scale + wi * 32;
            // Direct store (FP16 pieces): lane l writes its row's 128 columns as 16-byte vectors,
            // the C loads one group of 8 columns ahead.  Taken when the 128 columns are inside C,
            // the rows' starts 16-byte aligned and every scale 2^-(row + column scale) a normal
            // float; else the store through shared memory below.  (The BF16 folding form keeps
            // the shared-memory store: with C read, the direct store measured 0.56 ms against
            // 0.36 ms for it at 4096^3.)
            bool fast = F16 && c0 + 128 <= p.N && (p.ldc & 3) == 0 && ((uintptr_t)p.C & 15) == 0;
            int nsr = 0;
            if (F16) {   // non-finite lines have scale -100000: out of range
                nsr = -rs_w[lane];
                int lo = cs_w[lane], hi = lo;
#pragma unroll
                for (int j = 1; j < 4; j++) {
                    lo = min(lo, cs_w[lane + 32 * j]);
                    hi = max(hi, cs_w[lane + 32 * j]);
                }
                lo = __reduce_min_sync(0xffffffffu, lo);
                hi = __reduce_max_sync(0xffffffffu, hi);
                fast = fast && nsr - hi >= -126 && nsr - lo <= 127;
            }
            if (__all_sync(0xffffffffu, fast)) {
                const bool rc = reads_c(p), rowok = row0 + lane < p.M;
                float *crow = p.C + (row0 + lane) * p.ldc + c0;
                float4 cn0 = make_float4(0.f, 0.f, 0.f, 0.f), cn1 = cn0;
                if (rc && rowok) {
                    cn0 = ldg_v4(crow);
                    cn1 = ldg_v4(crow + 4);
                }
#pragma unroll
                for (int g = 0; g < 16; g++) {
                    const float cc[8] = {cn0.x, cn0.y, cn0.z, cn0.w, cn1.x, cn1.y, cn1.z, cn1.w};
                    if (g + 1 < 16 && rc && rowok) {   // issued before this group's stores (ordered asm)
                        cn0 = ldg_v4(crow + 8 * (g + 1));
                        cn1 = ldg_v4(crow + 8 * (g + 1) + 4);
                    }
                    float *o = total + 8 * g;   // the outputs replace their totals
                    if (F16) {
                        const int4 s0 = *reinterpret_cast<const int4 *>(cs_w + 8 * g);
                        const int4 s1 = *reinterpret_cast<const int4 *>(cs_w + 8 * g + 4);
                        const int sc[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
#pragma unroll
                        for (int j = 0; j < 8; j++) o[j] = epi_value(p, o[j] * pow2f(nsr - sc[j]), cc[j]);
                    } else {
#pragma unroll
                        for (int j = 0; j < 8; j++) o[j] = epi_value(p, o[j], cc[j]);
                    }
                    if (rowok) {
                        stg_v4(crow + 8 * g, make_float4(o[0], o[1], o[2], o[3]));
                        stg_v4(crow + 8 * g + 4, make_float4(o[4], o[5], o[6], o[7]));
                    }
                }
                continue;
            }
            float *stg = epi + wi * 32 * 17;
            const bool rc = reads_c(p);
            const int cl = lane & 15, rh = lane >> 4;   // this lane's column and row parity when storing
            // C in passes of 16 columns through shared memory: lane l holds row l's totals; after
            // the transpose lane l takes column l % 16 of rows l / 16, l / 16 + 2, ..., so each
            // load / store instruction covers two 64-byte row segments
            bool nf = false;
            const int64_t rows_left = p.M - row0;
#pragma unroll
            for (int ps = 0; ps < 8; ps++) {
#pragma unroll
                for (int j = 0; j < 16; j++) stg[lane * 17 + j] = total[16 * ps + j];
                __syncwarp();
                const int64_t col = c0 + 16 * ps + cl;
                const bool colok = col < p.N;
                const int cs = F16 ? cs_w[16 * ps + cl] : 0;
                float *cp = p.C + (row0 + rh) * p.ldc + col;
#pragma unroll
                for (int i8 = 0; i8 < 16; i8 += 8) {   // C loads eight at a time
                    float cin[8];
#pragma unroll
                    for (int i = i8; i < i8 + 8; i++)
                        cin[i - i8] = (rc && colok && 2 * i + rh < rows_left) ? cp[(int64_t)(2 * i) * p.ldc] : 0.f;
#pragma unroll
                    for (int i = i8; i < i8 + 8; i++) {
                        const int rr = 2 * i + rh;
                        float x = stg[rr * 17 + cl];
                        bool skip = false;
                        if (F16) {
                            const int sr = rs_w[rr];
                            skip = sr == kNonFiniteScale || cs == kNonFiniteScale;
                            x = mul_pow2f(x, -(sr + cs));
                        }
                        if (colok && rr < rows_left) {
                            if (skip) nf = true;
                            else cp[(int64_t)(2 * i) * p.ldc] = epi_value(p, x, cin[i - i8]);
                        }
                    }
                }
                __syncwarp();
            }
            if (F16 && __any_sync(0xffffffffu, nf)) {   // outputs whose line holds an Inf or a NaN
                for (int ps = 0; ps < 8; ps++) {
                    const int64_t col = c0 + 16 * ps + cl;
                    if (col >= p.N) continue;
                    const int cs = cs_w[16 * ps + cl];
                    for (int i = 0; i < 16; i++) {
                        const int rr = 2 * i + rh;
                        if (row0 + rr < p.M && (rs_w[rr] == kNonFiniteScale || cs == kNonFiniteScale))
                            store_recomputed(p, row0 + rr, col);
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
    if (threadIdx.x == 0 && p.done) atomicAdd(p.done, 1ull);   // last: this CTA is done
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

static gb_status two_pass(const GemmArgs &g, int np, int fold_kb, bool f16);

// Accumulator chunk in k-blocks of 32 (0: one accumulator over all of K):
// the call's accum_k (values of K, < 0 none), else the environment variable
// (k-blocks, for measurement), else the form's default.
static int chunk_kb(const GemmArgs &g, const char *env, int dflt) {
    if (g.accum_k < 0) return 0;
    if (g.accum_k > 0) return (int)((g.accum_k + 31) / 32);
    const char *v = getenv(env);
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
    return two_pass(g, 2, chunk_kb(g, "GB_BF16X3_FOLD", 0), false);
}

gb_status launch_sgemm_bf16x6(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    if (g.M > 0x7fffffff / 2 || g.N > 0x7fffffff / 2 || g.K > 0x7fffffff / 2)
        return set_status(GB_ERR_UNSUPPORTED, "bf16x6: dimension too large");
    return two_pass(g, 3, chunk_kb(g, "GB_BF16X6_CHUNK", 8), false);
}

gb_status launch_sgemm_fp16x3(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    if (g.M > 0x7fffffff / 2 || g.N > 0x7fffffff / 2 || g.K > 0x7fffffff / 2)
        return set_status(GB_ERR_UNSUPPORTED, "fp16x3: dimension too large");
    return two_pass(g, 2, chunk_kb(g, "GB_FP16X3_FOLD", 4), true);
}

// ------------------------------------------------------------ stream state
// Per (device, stream): a counter of finished GEMM CTAs (a slot of a static
// device array, so tracking needs no allocation), how many CTAs the stream's
// GEMMs launched so far, the byte range of the last GEMM's C and the
// workspace half its pieces are in.  A split pass is launched beside the
// previous GEMM only when that GEMM was this library's, this call's A and B
// do not overlap its C, and the two halves fit; split_entry_guard covers
// work the caller queued in between.
constexpr int kDoneSlots = 1024;
static __device__ unsigned long long g_gemm_done[kDoneSlots];
static __device__ unsigned long long g_scan_done[kDoneSlots];   // finished FP16 scan CTAs

struct StreamState {
    int dev;
    void *stream;
    int slot;                    // index into g_gemm_done / g_scan_done, -1: none left
    unsigned long long launched; // CTAs of this stream's GEMMs launched so far
    bool valid;                  // the stream's last two-pass GEMM is known
    uintptr_t c_lo, c_hi;        // its C
    unsigned parity;             // its workspace half
    unsigned long long scanned;  // CTAs of this stream's FP16 scans launched so far
    unsigned gen;                // generation of its last FP16 scan (captured scans use 1)
};
static std::mutex g_tp_mu;
static std::vector<StreamState> g_tp;
static unsigned long long *g_done_base[64] = {nullptr};

static StreamState &stream_state(int dev, void *stream) {
    int used = 0;
    for (auto &s : g_tp) {
        if (s.dev == dev && s.stream == stream) return s;
        if (s.dev == dev) used++;
    }
    g_tp.push_back(StreamState{dev, stream, used < kDoneSlots ? used : -1, 0ull, false, 0, 0, 0u, 0ull, 1u});
    return g_tp.back();
}

static unsigned long long *g_scan_base[64] = {nullptr};

static unsigned long long *scan_counter(int dev, int slot) {
    if (slot < 0 || dev < 0 || dev >= 64) return nullptr;
    if (!g_scan_base[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scan_done) != cudaSuccess || !p) {
            cudaGetLastError();
            return nullptr;
        }
        g_scan_base[dev] = (unsigned long long *)p;
    }
    return g_scan_base[dev] + slot;
}

static unsigned long long *done_counter(int dev, int slot) {
    if (slot < 0 || dev < 0 || dev >= 64) return nullptr;
    if (!g_done_base[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_gemm_done) != cudaSuccess || !p) {
            cudaGetLastError();
            return nullptr;
        }
        g_done_base[dev] = (unsigned long long *)p;
    }
    return g_done_base[dev] + slot;
}

// Bytes [lo, hi) spanned by a rows x cols operand stored with leading
// dimension ld (transposed storage: cols x rows).
static void span(const void *p, bool trans, int64_t rows, int64_t cols, int64_t ld, int64_t elem, uintptr_t &lo,
                 uintptr_t &hi) {
    const int64_t sr = trans ? cols : rows, sc = trans ? rows : cols;
    lo = (uintptr_t)p;
    hi = lo + (uintptr_t)(((sr - 1) * ld + sc) * elem);
}

template <int NP, int BN, bool FOLD, bool F16, int EW>
static gb_status two_pass_launch(const GemmArgs &g, const PieceMaps &maps, int64_t kp, const EpiParams &base,
                                 int *grid_out) {
    using CF = TwoPass<NP, BN, EW>;
    static std::atomic<uint64_t> attr{0};
    if (device_setup_needed(attr)) {
        GB_CUDA_TRY(cudaFuncSetAttribute(bf16x3_gemm_kernel<NP, BN, FOLD, F16, EW>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM_BYTES));
        device_setup_done(attr);
    }
    const int tiles_m = (int)ceil_div(g.M, BM), tiles_n = (int)ceil_div(g.N, BN);
    const int tiles = tiles_m * tiles_n;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    // half-tile tail when the last wave is at most half full (whole tiles
    // would leave most of the GPU idle for a tile time); GB_BF16X3_HALF=0 off.
    // The folding form keeps whole tiles unless GB_BF16X3_HALF=1: its halves
    // fold and store as often as whole tiles for half the MMA work, and the
    // FP16X3 call at 4096^3 measured 0.383 ms with them against 0.368 without.
    int half_start = tiles;
    {
        const char *e = getenv("GB_BF16X3_HALF");
        const int rem = tiles % grid;
        const bool on = FOLD ? (EW == 8 && e && e[0] == '1') : !(e && e[0] == '0');
        if (BN == 256 && on && rem > 0 && 2 * rem <= grid) half_start = tiles - rem;
    }
    EpiParams p = base;
    p.num_kb = (int)(kp / BK);
    p.tiles_m = tiles_m;
    p.tiles_n = tiles_n;
    p.chunk_kb = FOLD ? (p.chunk_kb > 0 ? p.chunk_kb : p.num_kb) : 1;
    p.half_start = half_start;
    bf16x3_gemm_kernel<NP, BN, FOLD, F16, EW><<<grid, CF::NT, CF::SMEM_BYTES, g.stream>>>(maps, p);
    GB_LAUNCH_CHECK("bf16x3_gemm_kernel");
    *grid_out = grid;
    return ok();
}

template <bool F16>
static gb_status gemm_launch(const GemmArgs &g, int np, int fold_kb, const PieceMaps &maps, int64_t kp,
                             const EpiParams &p, int *grid) {
    if constexpr (!F16) {   // three pieces are BF16 only
        if (np == 3)
            return fold_kb > 0 ? two_pass_launch<3, 128, true, false, 4>(g, maps, kp, p, grid)
                               : two_pass_launch<3, 128, false, false, 4>(g, maps, kp, p, grid);
    }
    if constexpr (F16) {   // always the wide folding form (fold_kb 0: one chunk over all of K)
        return two_pass_launch<2, 256, true, true, 8>(g, maps, kp, p, grid);
    } else {
        return fold_kb > 0 ? two_pass_launch<2, 256, true, false, 8>(g, maps, kp, p, grid)
                           : two_pass_launch<2, 256, false, false, 4>(g, maps, kp, p, grid);
    }
}

// Split pass (NP 16-bit pieces per operand, K-major) + MMA kernel; fold_kb >
// 0 selects the folding form with that accumulator chunk (in k-blocks of 32);
// f16: FP16 pieces of scaled lines (a max-exponent scan first).
static gb_status two_pass(const GemmArgs &g, int np, int fold_kb, bool f16) {
    if (f16 && np != 2) return set_status(GB_ERR_UNSUPPORTED, "fp16 pieces: two per value");
    const int64_t kp = ceil_div(g.K, 64) * 64;   // multiple of BK, zero-padded
    const size_t a_bytes = (size_t)g.M * kp * 2, b_bytes = (size_t)g.N * kp * 2;
    const size_t piece_bytes = (np * (a_bytes + b_bytes) + 255) / 256 * 256;
    const size_t pieces = piece_bytes;
    // The buffer is [half 0 | half 1], the same for every call of any form (the halves move only
    // when the buffer grows, which first drains its stream).  Calls alternate between the halves,
    // so a split may run beside the previous GEMM; one half when two do not fit in 16 GiB.
    const char *pe = getenv("GB_BF16X3_PDL");
    const bool pdl_env = !(pe && pe[0] == '0');
    const size_t want = pieces <= (size_t(8) << 30) ? 2 * pieces : pieces;
    unsigned seq_unused = 0;
    size_t ws_size = 0;
    uint8_t *ws = (uint8_t *)workspace(want, g.stream, &seq_unused, &ws_size);
    if (!ws) return (gb_status)gb_get_last_status();
    const size_t half = ws_size / 2 / 256 * 256;
    const bool two_halves = half >= pieces;
    // FP16 form: the line maxima, [half 0 | half 1] of lm_cap entries, in a buffer of their own
    unsigned long long *lm_base = nullptr;
    size_t lm_cap = 0;
    if (f16) {
        size_t lm_size = 0;
        lm_base = (unsigned long long *)linemax_buffer((size_t)16 * (g.M + g.N), g.stream, &lm_size);
        if (!lm_base) return (gb_status)gb_get_last_status();
        lm_cap = lm_size / 16;
    }
    int *err = error_word();
    if (!err) return set_status(GB_ERR_OOM, "bf16x3: no device error word");
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    static std::atomic<uint64_t> carve{0};
    if (device_setup_needed(carve)) {   // the GEMM's shared-memory configuration, so a split fits beside it
        GB_CUDA_TRY(cudaFuncSetAttribute(split_vec_kernel<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        GB_CUDA_TRY(cudaFuncSetAttribute(split_kernel<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        GB_CUDA_TRY(cudaFuncSetAttribute(split_vec_kernel<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        GB_CUDA_TRY(cudaFuncSetAttribute(split_kernel<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        GB_CUDA_TRY(cudaFuncSetAttribute(maxbits_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        device_setup_done(carve);
    }

    // Launches captured into a graph run whenever the graph is replayed, so the host cannot
    // count their CTAs: a captured call neither tracks nor overlaps.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    GB_CUDA_TRY(cudaStreamIsCapturing(g.stream, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;

    // the stream's state and this call's launches as one step
    std::lock_guard<std::mutex> lk(g_tp_mu);
    StreamState &st = stream_state(dev, g.stream);
    unsigned long long *done = capturing ? nullptr : done_counter(dev, st.slot);
    uintptr_t alo, ahi, blo, bhi, clo, chi;
    span(g.A, g.ta, g.M, g.K, g.lda, 4, alo, ahi);
    span(g.B, g.tb, g.K, g.N, g.ldb, 4, blo, bhi);
    span(g.C, false, g.M, g.N, g.ldc, 4, clo, chi);
    const bool pdl = pdl_env && two_halves && done != nullptr && st.valid &&
                     (ahi <= st.c_lo || alo >= st.c_hi) && (bhi <= st.c_lo || blo >= st.c_hi);
    const unsigned parity = two_halves ? (st.parity ^ 1u) : 0u;
    uint8_t *pw = ws + (size_t)parity * half;
    uint16_t *ap[3], *bp[3];
    for (int i = 0; i < np; i++) {
        ap[i] = (uint16_t *)(pw + i * a_bytes);
        bp[i] = (uint16_t *)(pw + np * a_bytes + i * b_bytes);
    }
    unsigned long long *bits = f16 ? lm_base + (size_t)parity * lm_cap : nullptr;   // op(A) rows, op(B) columns
    const unsigned long long *gdone = pdl ? done : nullptr;
    const unsigned long long expect = st.launched;
    unsigned long long *scan_done = f16 && done ? scan_counter(dev, st.slot) : nullptr;
    unsigned long long scan_expect = 0;
    unsigned gen = 1;
    if (f16 && !capturing) {
        if (st.gen >= 0xfffffff0u) {   // generations run out: clear the maxima and start again
            GB_CUDA_TRY(cudaMemsetAsync(lm_base, 0, 2 * lm_cap * sizeof(unsigned long long), g.stream));
            st.gen = 1;
        }
        gen = ++st.gen;   // > 1: above what a captured scan (generation 1) leaves
    }

    cudaLaunchAttribute pdl_attr[1];
    pdl_attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl_attr[0].val.programmaticStreamSerializationAllowed = 1;
    const bool vec = g.lda % 4 == 0 && g.ldb % 4 == 0 && (uintptr_t)g.A % 16 == 0 && (uintptr_t)g.B % 16 == 0;

    if (f16) {   // largest |x| of every row of op(A) and column of op(B)
        // a captured scan replays with its generation fixed: it clears its entries first
        if (capturing) GB_CUDA_TRY(cudaMemsetAsync(bits, 0, (size_t)(g.M + g.N) * 8, g.stream));
        ScanArgs sc;
        memset(&sc, 0, sizeof(sc));
        sc.K = g.K;
        sc.vec = vec ? 1 : 0;
        sc.gen = gen;
        sc.done = gdone;
        sc.expect = expect;
        sc.scan_done = scan_done;
        const int64_t tk = ceil_div(g.K, 256);   // a scan CTA covers 64 lines x 256 k
        sc.op[0] = ScanOp{(const float *)g.A, g.lda, g.M, tk, ceil_div(g.M, 64) * tk, g.ta ? 1 : 0, bits};
        sc.op[1] = ScanOp{(const float *)g.B, g.ldb, g.N, tk, ceil_div(g.N, 64) * tk, g.tb ? 0 : 1, bits + g.M};
        const int64_t blocks = sc.op[0].tiles + sc.op[1].tiles;
        if (blocks > 0x7fffffff) return set_status(GB_ERR_UNSUPPORTED, "fp16x3: operands too large");
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)blocks);
        cfg.blockDim = dim3(256);
        cfg.stream = g.stream;
        cfg.attrs = pdl_attr;
        cfg.numAttrs = pdl ? 1 : 0;
        GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, maxbits_kernel, sc));
        GB_LAUNCH_CHECK("fp16x3 scan");
        if (scan_done) {
            st.scanned += (unsigned long long)blocks;
            scan_expect = st.scanned;
        }
    }

    // split: op(A)(m, k) = ta ? A[k*lda + m] : A[m*lda + k]
    //        op(B)^T(n, k) = op(B)(k, n) = tb ? B[n*ldb + k] : B[k*ldb + n]
    if (vec) {
        SplitArgs sa;
        memset(&sa, 0, sizeof(sa));
        sa.K = g.K; sa.kp = kp; sa.np = np; sa.done = gdone; sa.expect = expect;
        sa.scan_done = scan_done; sa.scan_expect = scan_expect; sa.err = err;
        sa.op[0] = SplitOp{(const float *)g.A, g.lda, g.M, kp / 64, ceil_div(g.M, 64) * (kp / 64), g.ta ? 1 : 0,
                           {ap[0], ap[1], np == 3 ? ap[2] : nullptr}, bits};
        sa.op[1] = SplitOp{(const float *)g.B, g.ldb, g.N, kp / 64, ceil_div(g.N, 64) * (kp / 64), g.tb ? 0 : 1,
                           {bp[0], bp[1], np == 3 ? bp[2] : nullptr}, f16 ? bits + g.M : nullptr};
        const int64_t blocks = sa.op[0].tiles + sa.op[1].tiles;
        if (blocks > 0x7fffffff) return set_status(GB_ERR_UNSUPPORTED, "bf16x3: operands too large");
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)blocks);
        cfg.blockDim = dim3(256);
        cfg.stream = g.stream;
        cfg.attrs = pdl_attr;
        cfg.numAttrs = pdl ? 1 : 0;
        if (f16) GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, split_vec_kernel<true>, sa));
        else GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, split_vec_kernel<false>, sa));
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
        const unsigned long long *mb = bits;
        const unsigned long long *no_scan = nullptr;
        if (f16)
            GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, split_kernel<true>, (const float *)g.A, g.lda, g.ta ? 1 : 0, g.M, g.K,
                                           kp, ap[0], ap[1], (uint16_t *)nullptr, mb, gdone, expect,
                                           (const unsigned long long *)scan_done, scan_expect, err));
        else
            GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, split_kernel<false>, (const float *)g.A, g.lda, g.ta ? 1 : 0, g.M,
                                           g.K, kp, ap[0], ap[1], np == 3 ? ap[2] : (uint16_t *)nullptr, mb, gdone,
                                           expect, no_scan, 0ull, err));
        GB_LAUNCH_CHECK("bf16x3 split A");
        const unsigned long long *mbB = f16 ? bits + g.M : nullptr;
        if (f16)
            split_kernel<true><<<sgB, 256, 0, g.stream>>>((const float *)g.B, g.ldb, g.tb ? 0 : 1, g.N, g.K, kp, bp[0],
                                                          bp[1], nullptr, mbB, nullptr, 0ull, nullptr, 0ull, err);
        else
            split_kernel<false><<<sgB, 256, 0, g.stream>>>((const float *)g.B, g.ldb, g.tb ? 0 : 1, g.N, g.K, kp,
                                                           bp[0], bp[1], np == 3 ? bp[2] : nullptr, nullptr, nullptr,
                                                           0ull, nullptr, 0ull, err);
        GB_LAUNCH_CHECK("bf16x3 split B");
    }

    const int bn = np == 3 ? 128 : 256;
    PieceMaps maps;
    memset(&maps, 0, sizeof(maps));
    bool okm = true;
    for (int i = 0; i < np; i++) {   // 2-byte elements, copied as they are (BF16 or FP16)
        okm = okm && make_tmap_bf16(&maps.a[i], ap[i], kp, g.M, kp * 2, BK, BM, 64);
        okm = okm && make_tmap_bf16(&maps.b[i], bp[i], kp, g.N, kp * 2, BK, bn, 64);
        okm = okm && make_tmap_bf16(&maps.bh[i], bp[i], kp, g.N, kp * 2, BK, bn / 2, 64);
    }
    if (!okm) return set_status(GB_ERR_CUDA, "bf16x3: cuTensorMapEncodeTiled failed");
    EpiParams p;
    memset(&p, 0, sizeof(p));
    p.C = (float *)g.C; p.M = g.M; p.N = g.N; p.ldc = g.ldc;
    p.alpha = (float)g.alpha; p.beta = (float)g.beta; p.semantics = g.semantics;
    p.err = err;
    p.chunk_kb = fold_kb;
    p.done = done;
    if (f16) {
        p.rowbits = bits; p.colbits = bits + g.M;
        p.A = (const float *)g.A; p.B = (const float *)g.B;
        p.lda = g.lda; p.ldb = g.ldb; p.K = g.K;
        p.ta = g.ta ? 1 : 0; p.tb = g.tb ? 1 : 0;
    }
    int grid = 0;
    gb_status s = f16 ? gemm_launch<true>(g, np, fold_kb, maps, kp, p, &grid)
                      : gemm_launch<false>(g, np, fold_kb, maps, kp, p, &grid);
    if (s != GB_OK) return s;
    if (done) st.launched += (unsigned long long)grid;
    st.valid = done != nullptr;
    st.c_lo = clo;
    st.c_hi = chi;
    st.parity = parity;
    return ok();
}

}  // namespace gb
