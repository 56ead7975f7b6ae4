// skinny.cu -- bandwidth-bound GEMM for a tiny N (thinB) or a tiny M (shortA).
//
// Replaces irr_thinB_{s,d}gemm_{NN,NT,TN,TT}
// (irr_thinB_sgemm_release_V1.2/device_code/irr_thinB_sgemm_kernel.c:2910,
// 3448, 4619, 5147; irr_thinB_dgemm_release_V0.0/.../irr_thinB_dgemm_kernel.c:
// 1607, 1903, 2587, 2869) and irr_shortA_{s,d}gemm_* (irr_shortA_sgemm_kernel.c:
// 1769, 2034, 2592, 2820; irr_shortA_dgemm_kernel.c:1607, 1849, 2431, 2665).
//
// Like the reference, shortA is computed as the transpose of a thinB problem
// (C^T = op(B)^T op(A)^T), so one pair of kernels streams the large operand
// ("X", rows x K) exactly once while the small one ("W", K x n, n <= 64) is
// staged per K slab in shared memory and read from L2 by every CTA.  The
// output is written through two strides, so C^T is never formed.
//
// Two kernels, by the layout of X:
//  * X row-major (K contiguous): each warp streams R rows along K with
//    16-byte loads (lane l holds k = 32*V*step + V*l .. +V-1), the next
//    step's loads in flight while the current step is multiplied by W read
//    straight from L1 (every CTA reads the same small W); lanes reduce with
//    shuffles at the end.  No shared memory, no block barriers.
//  * X K-major (rows contiguous): each thread owns groups of 4 consecutive
//    rows loaded 16 bytes at a time, W is staged per K slab in shared memory
//    and read by broadcast.
// Split-K over CTAs when the row count alone cannot fill the GPU; partial
// sums go to scratch and a second kernel applies alpha/beta.
#include "gb_common.cuh"
#include "sm100_ptx.cuh"

namespace gb {

bool make_tmap_f32(CUtensorMap *map, const void *base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                   uint32_t box_inner, uint32_t box_outer, bool sw128);

namespace {

constexpr int NT = 256;

struct SkParams {
    int64_t rows, K;                      // X is rows x K (logical)
    const void *X; int64_t ldx; int tx;   // tx: X stored transposed (K x rows)
    const void *W; int64_t ldw; int tw;   // W logical K x n; tw: stored n x K
    int n;                                // logical small dimension (<= NB)
    void *C; int64_t cs_r, cs_c;          // C(r, j) at C[r*cs_r + j*cs_c]
    double alpha, beta;
    int semantics;
    int splits; int64_t kchunk;           // split-K
    int want_splits;                      // requested split count (0: the planner's choice)
    void *part;                           // splits x rows x NB partials (split-K only)
    void *wpieces;                        // BF16 pieces of W (tensor-core form only)
};

// row-major X: R rows per warp, lane l covers k = 32*V*step + V*l .. +V-1
template <typename T, int NB>
struct RowCfg {
    static constexpr int V = 16 / (int)sizeof(T);   // elements per 16-byte load
    static constexpr int KS = 32 * V;               // k per warp step
    static constexpr int R = NB <= 8 ? 8 : NB <= 16 ? 4 : 1;
    static constexpr int BR = (NT / 32) * R;        // rows per CTA
};

// K-major X: each thread owns G groups of VR consecutive rows (one vector
// load across rows), sized so R * NB stays near 64 accumulators; a CTA
// covers NT * VR * G rows
template <typename T, int NB>
struct ColCfg {
    static constexpr int R0 = (64 * 4 / (int)sizeof(T)) / NB;      // accumulator budget in rows
    static constexpr int VMAX = 16 / (int)sizeof(T);
    static constexpr int VR = R0 >= VMAX ? VMAX : (R0 >= 2 ? 2 : 1);   // rows per vector load
    static constexpr int G = R0 / VR >= 2 ? 2 : 1;
    static constexpr int R = VR * G;                // rows per thread
    static constexpr int SLAB = 32768 / (int)sizeof(T) / NB;
    static constexpr int BR = NT * R;
    static constexpr int U = 4;                     // k unroll (loads in flight)
};

template <typename T>
__device__ __forceinline__ void epilogue_store(const SkParams &p, int64_t r, int j, T acc) {
    T *cp = (T *)p.C + r * p.cs_r + (int64_t)j * p.cs_c;
    T v = (T)p.alpha * acc;
    if (p.semantics == GB_SEM_BLAS) {
        if (p.beta != 0.0) v = fma((T)p.beta, *cp, v);
    } else if (p.semantics == GB_SEM_SCALAR_BETA) {
        v = v + (T)p.beta;
    } else {
        v = *cp + (v + (T)p.beta);
    }
    *cp = v;
}

// Stage W[k0 .. k0+cnt) x NB into shared memory, zero beyond kend / n.
// Threads walk the shared-memory index e (conflict-free stores); decode(e)
// gives the (kk, j) element it holds.  W is small and L2-resident, so the
// strided global reads this implies are cheap.
template <typename T, int NB, typename Decode>
__device__ __forceinline__ void stage_w(const SkParams &p, T *Ws, int64_t k0, int cnt, int64_t kend, Decode decode) {
    const T *W = (const T *)p.W;
    for (int e = threadIdx.x; e < cnt * NB; e += NT) {
        int kk, j;
        decode(e, kk, j);
        const int64_t k = k0 + kk;
        T v = T(0);
        if (j < p.n && k < kend) v = p.tw ? W[(int64_t)j * p.ldw + k] : W[k * p.ldw + j];
        Ws[e] = v;
    }
}

template <typename T, int V>
struct VecT;
template <>
struct VecT<float, 4> {
    __device__ static void load(const float *p, float *o) {
        float4 v = __ldg(reinterpret_cast<const float4 *>(p));
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
};
template <>
struct VecT<double, 2> {
    __device__ static void load(const double *p, double *o) {
        double2 v = __ldg(reinterpret_cast<const double2 *>(p));
        o[0] = v.x; o[1] = v.y;
    }
};
template <>
struct VecT<float, 2> {
    __device__ static void load(const float *p, float *o) {
        float2 v = __ldg(reinterpret_cast<const float2 *>(p));
        o[0] = v.x; o[1] = v.y;
    }
};
template <typename T>
struct VecT<T, 1> {
    __device__ static void load(const T *p, T *o) { o[0] = __ldg(p); }
};

// X rows [r0, r0+R) at k = kb .. kb+V-1 into xv (zero beyond rows / kend).
template <typename T, int R, int V, bool VEC>
__device__ __forceinline__ void load_x_rows(const SkParams &p, const T *X, int64_t r0, int64_t kb, int64_t kend,
                                            T (&xv)[R][V]) {
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int64_t row = r0 + i;
        const T *xp = X + row * p.ldx + kb;
        if (VEC && row < p.rows && kb + V <= kend) {
            VecT<T, V>::load(xp, xv[i]);
        } else {
#pragma unroll
            for (int q = 0; q < V; q++) xv[i][q] = (row < p.rows && kb + q < kend) ? xp[q] : T(0);
        }
    }
}

// acc += X(rows, kb..kb+V-1) * W(kb..kb+V-1, :).  W comes from L1 / L2 (it
// is small and every CTA reads it): 16-byte loads along W's contiguous
// dimension when WVEC, else guarded scalar loads.
template <typename T, int NB, int R, int V, bool WVEC>
__device__ __forceinline__ void fma_step(const SkParams &p, const T *W, int64_t kb, int64_t kend, const T (&xv)[R][V],
                                         T (&acc)[R][NB]) {
    if (WVEC && kb + V <= kend) {
        if (p.tw) {            // W stored n x K: V consecutive k of column j
#pragma unroll
            for (int j = 0; j < NB; j++) {
                T w[V];
                VecT<T, V>::load(W + (int64_t)j * p.ldw + kb, w);
#pragma unroll
                for (int q = 0; q < V; q++)
#pragma unroll
                    for (int i = 0; i < R; i++) acc[i][j] = fma(xv[i][q], w[q], acc[i][j]);
                if (NB > 16 && (j & 15) == 15) asm volatile("" ::: "memory");   // bound load hoisting
            }
        } else {               // W stored K x n (n == NB): row k holds NB consecutive values
#pragma unroll
            for (int q = 0; q < V; q++) {
#pragma unroll
                for (int j0 = 0; j0 < NB; j0 += V) {
                    T w[V];
                    VecT<T, V>::load(W + (kb + q) * p.ldw + j0, w);
#pragma unroll
                    for (int jj = 0; jj < V; jj++)
#pragma unroll
                        for (int i = 0; i < R; i++) acc[i][j0 + jj] = fma(xv[i][q], w[jj], acc[i][j0 + jj]);
                    if (NB > 16 && (j0 & 15) == 16 - V) asm volatile("" ::: "memory");
                }
            }
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < V; q++) {
        const int64_t k = kb + q;
#pragma unroll
        for (int j = 0; j < NB; j++) {
            T w = T(0);
            if (k < kend && j < p.n) w = p.tw ? __ldg(W + (int64_t)j * p.ldw + k) : __ldg(W + k * p.ldw + j);
#pragma unroll
            for (int i = 0; i < R; i++) acc[i][j] = fma(xv[i][q], w, acc[i][j]);
        }
    }
}

template <typename T, int NB, bool VEC, bool WVEC>
__global__ void __launch_bounds__(NT) skinny_rows_kernel(SkParams p) {
    using C = RowCfg<T, NB>;
    constexpr int V = C::V, KS = C::KS, R = C::R;
    const T *X = (const T *)p.X, *W = (const T *)p.W;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int64_t r0 = (int64_t)blockIdx.x * C::BR + warp * R;
    const int split = blockIdx.y;
    const int64_t kbeg = (int64_t)split * p.kchunk;
    const int64_t kend = kbeg + p.kchunk < p.K ? kbeg + p.kchunk : p.K;

    T acc[R][NB];
#pragma unroll
    for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < NB; j++) acc[i][j] = T(0);

    // two register buffers, the next step's X loads in flight while the
    // current step's FMAs run
    const int64_t nsteps = (kend - kbeg + KS - 1) / KS;
    T xa[R][V], xb[R][V];
    const int64_t kl = kbeg + lane * V;
    if (nsteps > 0) load_x_rows<T, R, V, VEC>(p, X, r0, kl, kend, xa);
    int64_t st = 0;
    for (; st + 1 < nsteps; st += 2) {
        load_x_rows<T, R, V, VEC>(p, X, r0, kl + (st + 1) * KS, kend, xb);
        fma_step<T, NB, R, V, WVEC>(p, W, kl + st * KS, kend, xa, acc);
        if (st + 2 < nsteps) load_x_rows<T, R, V, VEC>(p, X, r0, kl + (st + 2) * KS, kend, xa);
        fma_step<T, NB, R, V, WVEC>(p, W, kl + (st + 1) * KS, kend, xb, acc);
    }
    if (st < nsteps) fma_step<T, NB, R, V, WVEC>(p, W, kl + st * KS, kend, xa, acc);

#pragma unroll
    for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < NB; j++) {
            T v = acc[i][j];
#pragma unroll
            for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            acc[i][j] = v;
        }
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int64_t row = r0 + i;
        if (row >= p.rows) continue;
#pragma unroll
        for (int j = 0; j < NB; j++) {
            if ((j & 31) != lane) continue;
            if (p.splits > 1)
                ((T *)p.part)[((int64_t)split * p.rows + row) * NB + j] = acc[i][j];
            else if (j < p.n)
                epilogue_store<T>(p, row, j, acc[i][j]);
        }
    }
}

template <typename T, int NB, bool VEC>
__global__ void __launch_bounds__(NT) skinny_cols_kernel(SkParams p) {
    using C = ColCfg<T, NB>;
    constexpr int VR = C::VR, G = C::G, R = C::R, U = C::U;
    __shared__ __align__(16) T Ws[C::SLAB * NB];   // [k][j], read by broadcast
    const T *X = (const T *)p.X;
    const int tid = threadIdx.x;
    const int64_t cta0 = (int64_t)blockIdx.x * C::BR;
    const int split = blockIdx.y;
    const int64_t kbeg = (int64_t)split * p.kchunk;
    const int64_t kend = kbeg + p.kchunk < p.K ? kbeg + p.kchunk : p.K;
    // rows of group g: cta0 + (g*NT + tid)*VR .. +VR-1 (consecutive threads, consecutive 16-byte chunks)
    T acc[R][NB];
#pragma unroll
    for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < NB; j++) acc[i][j] = T(0);

    for (int64_t k0 = kbeg; k0 < kend; k0 += C::SLAB) {
        const int cnt = (int)((kend - k0) < C::SLAB ? (kend - k0) : C::SLAB);
        __syncthreads();
        stage_w<T, NB>(p, Ws, k0, C::SLAB, kend, [](int e, int &kk, int &j) {
            kk = e / NB;
            j = e - kk * NB;
        });
        __syncthreads();
        for (int kk = 0; kk < cnt; kk += U) {
            T x[U][R];
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int g = 0; g < G; g++) {
                    const int64_t rb = cta0 + ((int64_t)g * NT + tid) * VR;
                    const T *xp = X + (k0 + kk + u) * p.ldx + rb;
                    const bool kin = kk + u < cnt;
                    if (VEC && kin && rb + VR <= p.rows) {
                        VecT<T, VR>::load(xp, &x[u][g * VR]);
                    } else {
#pragma unroll
                        for (int v = 0; v < VR; v++) x[u][g * VR + v] = (kin && rb + v < p.rows) ? xp[v] : T(0);
                    }
                }
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int j = 0; j < NB; j++) {
                    const T w = Ws[(kk + u) * NB + j];   // beyond cnt: zero-staged
#pragma unroll
                    for (int i = 0; i < R; i++) acc[i][j] = fma(x[u][i], w, acc[i][j]);
                }
        }
    }

#pragma unroll
    for (int g = 0; g < G; g++)
#pragma unroll
        for (int v = 0; v < VR; v++) {
            const int i = g * VR + v;
            const int64_t row = cta0 + ((int64_t)g * NT + tid) * VR + v;
            if (row >= p.rows) continue;
            if (p.splits > 1) {
                T *part = (T *)p.part + ((int64_t)split * p.rows + row) * NB;
#pragma unroll
                for (int j = 0; j < NB; j++) part[j] = acc[i][j];
                continue;
            }
#pragma unroll
            for (int j = 0; j < NB; j++)
                if (j < p.n) epilogue_store<T>(p, row, j, acc[i][j]);
        }
}

// ---------------------------------------------------------------------------
// FP32, n <= 8: the large operand streamed by TMA.  Persistent CTAs (one per
// SM) walk units of BR rows x one K range; a producer warp keeps the stages
// (BR x 32 X values plus the matching 32 x NS slice of W) in flight, so the
// memory system sees ~200 KB of outstanding reads per SM whatever the
// register use; consumer threads own R rows each and run the whole K range
// of them (FMAs in k order, no cross-thread reduction).
// X row-major arrives as 128-byte-swizzled 32-float rows (conflict-free
// 16-byte reads across 8 consecutive rows); X K-major as [32 k][256 rows]
// boxes.  W is read by broadcast in either of its layouts; a broadcast read
// still costs a shared-memory wavefront per value, so for n = 8 each thread
// keeps R = 4 rows to share every W value across four rows (that keeps the
// shared-memory pipe near half load at full HBM rate), for n <= 4 one row.
// Partial sums of a split K range go to scratch for skinny_reduce_kernel.
namespace thin {

constexpr int BK = 32;
constexpr int WS = 1024;            // W slice (BK x NS floats), padded to keep stages 1 KB aligned

template <int R>
struct TCfg {
    static constexpr int NCW = R == 1 ? 8 : 4;                 // consumer warps
    static constexpr int NTH = (NCW + 1) * 32;
    static constexpr int BR = NCW * 32 * R;                    // rows per unit: 256 or 512
    static constexpr int NBOX = BR / 256;                      // TMA boxes of 256 rows per stage
    static constexpr int XS = BR * BK * 4;                     // 32 or 64 KB
    static constexpr int STAGE = XS + WS;
    static constexpr int STAGES = R == 1 ? 6 : 3;
    static constexpr int SMEM = STAGES * STAGE + 1024 /*align*/ + 256 /*barriers*/;
};

template <int NS>
__host__ __device__ constexpr int rows_per_thread() { return NS > 4 ? 4 : 1; }

// Row-major X whose leading dimension is not a multiple of 4 floats is taken
// in four row classes r = 4i + c, each with its own 16-byte aligned tensor
// map (base X + c*ldx - d_c, row stride 4*ldx, coordinate x holding
// k = x - d_c); W is then read from a packed copy Wp[k + 32][NS] whose row
// coordinate absorbs the shift, and the values at k < 0 (the previous row's
// tail) are zeroed.
struct TParams {
    int64_t rows, K;
    int n, splits, kchunk_kb, nkb;
    int rstride, woff;                    // 4 / 32 with row classes (packed W), else 1 / 0
    int64_t cls_rows[4];
    int cls_delta[4];
    int cls_u0[5];
    void *C; int64_t cs_r, cs_c;
    float alpha, beta;
    int semantics;
    float *part;
    int *err;
};

struct TMaps {
    CUtensorMap x[4], w;
};

__device__ __forceinline__ void tunit(const TParams &p, int u, int &c, int &rt, int &sp) {
    c = 0;
    while (c < 3 && u >= p.cls_u0[c + 1]) c++;
    const int v = u - p.cls_u0[c];
    rt = v / p.splits;
    sp = v - rt * p.splits;
}

template <int NS, bool XCOLS, bool WT>
__global__ void __launch_bounds__(TCfg<rows_per_thread<NS>()>::NTH, 1)
    thin_tma_kernel(const __grid_constant__ TMaps maps, TParams p) {
    constexpr int R = rows_per_thread<NS>();
    using CF = TCfg<R>;
    constexpr int NCW = CF::NCW, BR = CF::BR, STAGES = CF::STAGES, STAGE = CF::STAGE, XS = CF::XS;
    constexpr int TPR = NCW * 32;   // threads per row slot
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE);
    uint64_t *empty = full + STAGES;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int nkb = p.nkb;
    const int units = p.cls_u0[4];
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], NCW);
        }
        ptx::fence_mbar_init();
    }
    __syncthreads();

    if (warp == NCW) {   // producer
        if (lane == 0) {
            int g = 0;
            for (int u = blockIdx.x; u < units; u += gridDim.x) {
                int c, rt, sp;
                tunit(p, u, c, rt, sp);
                const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
                const int r0 = rt * BR;
                for (int kb = kb0; kb < kb1; kb++, g++) {
                    const int s = g % STAGES;
                    if (g >= STAGES && !ptx::mbar_wait(&empty[s], ((g / STAGES) & 1) ^ 1, p.err, 41)) return;
                    uint8_t *st = smem + s * STAGE;
                    ptx::mbar_arrive_expect_tx(&full[s], XS + BK * NS * 4);
#pragma unroll
                    for (int bx = 0; bx < CF::NBOX; bx++) {
                        if (XCOLS) ptx::tma_load_2d(st + bx * 32768, &maps.x[c], &full[s], r0 + bx * 256, kb * BK);
                        else ptx::tma_load_2d(st + bx * 32768, &maps.x[c], &full[s], kb * BK, r0 + bx * 256);
                    }
                    if (WT) ptx::tma_load_2d(st + XS, &maps.w, &full[s], kb * BK, 0);
                    else ptx::tma_load_2d(st + XS, &maps.w, &full[s], 0, kb * BK + p.woff - p.cls_delta[c]);
                }
            }
        }
        return;
    }

    // consumer thread t: rows r0 + t + i*TPR, i < R (row slot i: 32 consecutive rows per warp)
    const int t = threadIdx.x;
    int g = 0;
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        int c, rt, sp;
        tunit(p, u, c, rt, sp);
        const int kb0 = sp * p.kchunk_kb, kb1 = min(nkb, kb0 + p.kchunk_kb);
        const int delta = p.cls_delta[c];
        float acc[R][NS];
#pragma unroll
        for (int i = 0; i < R; i++)
#pragma unroll
            for (int j = 0; j < NS; j++) acc[i][j] = 0.f;
        bool go = true;
        for (int kb = kb0; kb < kb1; kb++, g++) {
            const int s = g % STAGES;
            if (!ptx::mbar_wait(&full[s], (g / STAGES) & 1, p.err, 42)) { go = false; break; }
            const uint8_t *st = smem + s * STAGE;
            const float *ws = reinterpret_cast<const float *>(st + XS);
            // two halves of 16 k, so the W reads the compiler hoists stay in registers
#pragma unroll 1
            for (int h = 0; h < BK; h += 16) {
                float x[R][16];
#pragma unroll
                for (int i = 0; i < R; i++) {
                    const int lr = t + i * TPR;                       // row within the unit
                    const uint8_t *box = st + (lr >> 8) * 32768;      // its 256-row TMA box
                    const int br = lr & 255;
                    if (XCOLS) {
                        const float *xs = reinterpret_cast<const float *>(box);
#pragma unroll
                        for (int kk = 0; kk < 16; kk++) x[i][kk] = xs[(h + kk) * 256 + br];
                    } else {
                        const uint8_t *row = box + br * 128;
#pragma unroll
                        for (int cc = 0; cc < 4; cc++) {
                            const float4 v = *reinterpret_cast<const float4 *>(row + (((h / 4 + cc) ^ (br & 7)) << 4));
                            x[i][4 * cc] = v.x; x[i][4 * cc + 1] = v.y; x[i][4 * cc + 2] = v.z; x[i][4 * cc + 3] = v.w;
                        }
                    }
                    if (kb == 0 && h == 0 && delta > 0) {   // coordinates below d_c are the previous row
#pragma unroll
                        for (int kk = 0; kk < 3; kk++)
                            if (kk < delta) x[i][kk] = 0.f;
                    }
                }
                if (WT) {   // ws[j][kk]
#pragma unroll
                    for (int k4 = 0; k4 < 16; k4 += 4) {
#pragma unroll
                        for (int j = 0; j < NS; j++) {
                            const float4 w = *reinterpret_cast<const float4 *>(ws + j * BK + h + k4);
#pragma unroll
                            for (int i = 0; i < R; i++) {
                                acc[i][j] = fmaf(x[i][k4], w.x, acc[i][j]);
                                acc[i][j] = fmaf(x[i][k4 + 1], w.y, acc[i][j]);
                                acc[i][j] = fmaf(x[i][k4 + 2], w.z, acc[i][j]);
                                acc[i][j] = fmaf(x[i][k4 + 3], w.w, acc[i][j]);
                            }
                        }
                    }
                } else {    // ws[kk][j]
#pragma unroll
                    for (int kk = 0; kk < 16; kk++) {
#pragma unroll
                        for (int j4 = 0; j4 < NS; j4 += 4) {
                            const float4 w = *reinterpret_cast<const float4 *>(ws + (h + kk) * NS + j4);
#pragma unroll
                            for (int i = 0; i < R; i++) {
                                acc[i][j4] = fmaf(x[i][kk], w.x, acc[i][j4]);
                                acc[i][j4 + 1] = fmaf(x[i][kk], w.y, acc[i][j4 + 1]);
                                acc[i][j4 + 2] = fmaf(x[i][kk], w.z, acc[i][j4 + 2]);
                                acc[i][j4 + 3] = fmaf(x[i][kk], w.w, acc[i][j4 + 3]);
                            }
                        }
                    }
                }
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&empty[s]);
        }
        if (!go) break;
#pragma unroll
        for (int i = 0; i < R; i++) {
            const int64_t ci = (int64_t)rt * BR + t + i * TPR;   // row within the class
            if (ci >= p.cls_rows[c]) continue;
            const int64_t row = ci * p.rstride + c;
            if (p.splits > 1) {
                float *pp = p.part + ((int64_t)sp * p.rows + row) * 8;
#pragma unroll
                for (int j = 0; j < NS; j++) pp[j] = acc[i][j];
                continue;
            }
            float *c = (float *)p.C + row * p.cs_r;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                if (j >= p.n) break;
                float *cp = c + (int64_t)j * p.cs_c;
                float v = p.alpha * acc[i][j];
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
}

}  // namespace thin

template <typename T, int NB>
__global__ void skinny_reduce_kernel(SkParams p) {
    const int64_t total = p.rows * p.n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = e / p.n;
        int j = (int)(e - r * p.n);
        T s = T(0);
        for (int sp = 0; sp < p.splits; sp++) s += ((const T *)p.part)[((int64_t)sp * p.rows + r) * NB + j];
        epilogue_store<T>(p, r, j, s);
    }
}

// Launch plan shared by the workspace path and the fixed-scratch path.
struct Plan {
    bool rows_kernel, vec, wvec;
    bool tma;                 // FP32 n <= 8 with TMA-compatible layouts: thin::thin_tma_kernel
    bool tc;                  // FP32 8 < n <= 64, K >= 64: 3xBF16 on the tensor cores (skinny_tc.cu)
    int64_t rtiles;
    size_t part_bytes;
    size_t w_bytes;           // scratch for the BF16 pieces of W (tc)
};

// TMA needs 16-byte aligned bases and row strides that are multiples of 16
// bytes; GB_SKINNY_TMA=0 turns the streamed kernel off (for measurement).
template <typename T, int NB>
bool tma_eligible(const SkParams &p) {
    if (sizeof(T) != 4 || NB != 8) return false;
    const char *e = getenv("GB_SKINNY_TMA");
    if (e && e[0] == '0') return false;
    // K-major X needs ldx % 4 == 0; row-major X any ldx (row classes); W any
    // layout (packed when the tensor map cannot read it in place)
    return p.K > 0 && p.rows < (int64_t(1) << 31) && p.K < (int64_t(1) << 30) && (p.ldx % 4 == 0 || !p.tx) &&
           (uintptr_t)p.X % 16 == 0;
}

// FFMA-TMA form: rows taken in four classes (row-major X, ldx % 4 != 0), and
// whether W is read from a packed copy
inline bool thin_classes(const SkParams &p) { return !p.tx && p.ldx % 4 != 0; }
inline bool thin_pack_w(const SkParams &p) {
    return thin_classes(p) || p.ldw % 4 != 0 || (uintptr_t)p.W % 16 != 0;
}
constexpr int64_t kWpOff = 32;   // packed W: row k at k + 32 (rows below and above K are zero)
inline int64_t thin_wp_rows(int64_t K) { return K + 2 * kWpOff + thin::BK; }

// The tensor-core form: X read by TMA (16-byte aligned base; any ldx -- four
// row or k-line classes when ldx % 4 != 0), any W layout (it is split into
// BF16 pieces first); GB_SKINNY_TC=0 turns it off.
template <typename T, int NB>
bool tc_eligible(const SkParams &p) {
    if (sizeof(T) != 4 || NB < 16 || p.n <= 8 || p.K < 64) return false;
    const char *e = getenv("GB_SKINNY_TC");
    if (e && e[0] == '0') return false;
    return p.rows < (int64_t(1) << 31) && p.K < (int64_t(1) << 30) && (uintptr_t)p.X % 16 == 0;
}

template <typename T, int NB>
gb_status make_plan(SkParams &p, Plan &pl, bool allow_tc = true) {
    pl.w_bytes = 0;
    pl.tc = allow_tc && tc_eligible<T, NB>(p);
    if (pl.tc) {
        // units of 128 rows (per row class) x a K range; split K until there are ~4 units per SM
        const bool classes = thin_tc_row_classes(p.tx, p.ldx);
        pl.tma = false;
        pl.rows_kernel = !p.tx;
        pl.vec = pl.wvec = true;
        pl.rtiles = ceil_div(p.rows, 128) + (classes ? 3 : 0);
        const int64_t nst = thin_tc_stages(p.K, classes);
        int splits = 1;
        while (pl.rtiles * splits < 4 * (int64_t)sm_count() && nst / (splits * 2) >= 8 && splits < 64) splits *= 2;
        if (p.want_splits > 0) splits = p.want_splits;
        const int64_t cst = ceil_div(nst, splits);
        p.kchunk = cst * 64;
        p.splits = (int)ceil_div(nst, cst);
        if (p.splits < 1) p.splits = 1;
        pl.part_bytes = p.splits > 1 ? (size_t)p.splits * p.rows * NB * sizeof(T) : 0;
        pl.w_bytes = thin_tc_wpieces_bytes(NB, p.K, classes);
        return ok();
    }
    pl.tma = tma_eligible<T, NB>(p);
    if (pl.tma) {
        // units of 256 rows x a K range; split K until there are ~4 units per SM
        pl.rows_kernel = !p.tx;
        pl.vec = pl.wvec = true;
        const int br = p.n > 4 ? thin::TCfg<4>::BR : thin::TCfg<1>::BR;
        const bool classes = thin_classes(p);
        pl.rtiles = ceil_div(p.rows, br) + (classes ? 3 : 0);
        const int64_t nkb = ceil_div(p.K + (classes ? 3 : 0), thin::BK);
        // split K until there are ~6 units per SM (tail balance of the persistent grid)
        int splits = 1;
        while (pl.rtiles * splits < 6 * (int64_t)sm_count() && nkb / (splits * 2) >= 16 && splits < 64) splits *= 2;
        if (p.want_splits > 0) splits = p.want_splits;
        const int64_t ckb = ceil_div(nkb, splits);
        p.kchunk = ckb * thin::BK;
        p.splits = (int)ceil_div(nkb, ckb);
        if (p.splits < 1) p.splits = 1;
        pl.part_bytes = p.splits > 1 ? (size_t)p.splits * p.rows * NB * sizeof(T) : 0;
        pl.w_bytes = thin_pack_w(p) ? (size_t)thin_wp_rows(p.K) * (p.n <= 4 ? 4 : 8) * sizeof(float) : 0;
        return ok();
    }
    pl.rows_kernel = !p.tx;
    const int64_t br = pl.rows_kernel ? RowCfg<T, NB>::BR : ColCfg<T, NB>::BR;
    const int64_t gran = pl.rows_kernel ? RowCfg<T, NB>::KS : ColCfg<T, NB>::U;
    pl.rtiles = ceil_div(p.rows, br);
    if (pl.rtiles > 0x7fffffff) return set_status(GB_ERR_UNSUPPORTED, "skinny: too many rows");
    // split K until the grid covers ~2 waves of the GPU
    const int64_t target = 2 * (int64_t)sm_count();
    int splits = 1;
    while (pl.rtiles * splits < target && p.K / (splits * 2) >= 256 && splits < 64) splits *= 2;
    if (p.want_splits > 0) splits = p.want_splits;
    p.kchunk = ceil_div(ceil_div(p.K, splits), gran) * gran;
    p.splits = (int)ceil_div(p.K, p.kchunk);
    if (p.splits < 1) p.splits = 1;
    constexpr int V = RowCfg<T, NB>::V;
    if (pl.rows_kernel) {
        pl.vec = (p.ldx % V == 0) && ((uintptr_t)p.X % 16 == 0);
        // W vector loads: n x K storage needs ldw % V == 0; K x n storage
        // additionally needs the full NB columns present (n == NB)
        pl.wvec = (p.ldw % V == 0) && ((uintptr_t)p.W % 16 == 0) && (p.tw || p.n == NB);
    } else {
        constexpr int VR = ColCfg<T, NB>::VR;
        pl.vec = (p.ldx % VR == 0) && ((uintptr_t)p.X % 16 == 0);
        pl.wvec = false;
    }
    pl.part_bytes = p.splits > 1 ? (size_t)p.splits * p.rows * NB * sizeof(T) : 0;
    return ok();
}

// W (logical K x n; tw: stored n x K) -> Wp[k + 32][j], ns columns, zero
// outside 0 <= k < K, j < n
__global__ void wpack_kernel(const float *__restrict__ W, int64_t ldw, int tw, int n, int64_t K, int64_t rows, int ns,
                             float *__restrict__ wp) {
    const int64_t total = rows * ns;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / ns, j = e - r * ns, k = r - kWpOff;
        float v = 0.f;
        if (j < n && k >= 0 && k < K) v = tw ? W[j * ldw + k] : W[k * ldw + j];
        wp[e] = v;
    }
}

template <int NS, bool XCOLS, bool WT>
gb_status launch_thin(const thin::TMaps &maps, const thin::TParams &tp, int grid, cudaStream_t st) {
    using CF = thin::TCfg<thin::rows_per_thread<NS>()>;
    static std::atomic<uint64_t> attr{0};
    if (device_setup_needed(attr)) {
        GB_CUDA_TRY(cudaFuncSetAttribute(thin::thin_tma_kernel<NS, XCOLS, WT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM));
        device_setup_done(attr);
    }
    thin::thin_tma_kernel<NS, XCOLS, WT><<<grid, CF::NTH, CF::SMEM, st>>>(maps, tp);
    GB_LAUNCH_CHECK("thin_tma_kernel");
    return ok();
}

template <typename T, int NB>
gb_status launch_plan(const SkParams &p, const Plan &pl, cudaStream_t st) {
    if (pl.tc) {
        ThinTcArgs a{p.rows, p.K, (const float *)p.X, p.ldx, p.tx, (const float *)p.W, p.ldw, p.tw, p.n, NB,
                     (float *)p.C, p.cs_r, p.cs_c, (float)p.alpha, (float)p.beta, p.semantics, p.splits, p.kchunk,
                     (float *)p.part, p.wpieces, st};
        gb_status s = launch_thin_tc(a);
        if (s != GB_OK) return s;
        if (p.splits > 1) {
            int blocks = (int)(ceil_div(p.rows * p.n, 256) < 4 * sm_count() ? ceil_div(p.rows * p.n, 256)
                                                                             : 4 * sm_count());
            skinny_reduce_kernel<T, NB><<<blocks, 256, 0, st>>>(p);
            GB_LAUNCH_CHECK("skinny_reduce_kernel");
        }
        return ok();
    }
    if (pl.tma) {
        const int ns = p.n <= 4 ? 4 : 8;
        const bool classes = thin_classes(p), pack = thin_pack_w(p);
        thin::TMaps maps;
        memset(&maps, 0, sizeof(maps));
        thin::TParams tp;
        memset(&tp, 0, sizeof(tp));
        tp.rows = p.rows; tp.K = p.K; tp.n = p.n; tp.splits = p.splits;
        tp.kchunk_kb = (int)(p.kchunk / thin::BK);
        tp.nkb = (int)ceil_div(p.K + (classes ? 3 : 0), thin::BK);
        tp.rstride = classes ? 4 : 1;
        tp.woff = pack ? (int)kWpOff : 0;
        bool okm = true;
        if (pack) {
            const int64_t rows = thin_wp_rows(p.K);
            const int blocks = (int)(ceil_div(rows * ns, 256) < 2 * sm_count() ? ceil_div(rows * ns, 256)
                                                                                : 2 * sm_count());
            wpack_kernel<<<blocks, 256, 0, st>>>((const float *)p.W, p.ldw, p.tw, p.n, p.K, rows, ns,
                                                 (float *)p.wpieces);
            GB_LAUNCH_CHECK("wpack_kernel");
            okm = make_tmap_f32(&maps.w, p.wpieces, (uint64_t)ns, (uint64_t)rows, (uint64_t)ns * 4, (uint32_t)ns,
                                thin::BK, false);
        } else {
            okm = p.tw ? make_tmap_f32(&maps.w, p.W, (uint64_t)p.K, (uint64_t)p.n, (uint64_t)p.ldw * 4, thin::BK,
                                       (uint32_t)ns, false)
                       : make_tmap_f32(&maps.w, p.W, (uint64_t)p.n, (uint64_t)p.K, (uint64_t)p.ldw * 4,
                                       (uint32_t)ns, thin::BK, false);
        }
        const int br = ns == 8 ? thin::TCfg<4>::BR : thin::TCfg<1>::BR;
        int u = 0;
        for (int c = 0; c < 4; c++) {
            tp.cls_u0[c] = u;
            int64_t rows_c = c == 0 ? p.rows : 0;
            int delta = 0;
            const float *base = (const float *)p.X;
            if (classes) {
                rows_c = p.rows > c ? (p.rows - c + 3) / 4 : 0;
                delta = (int)((c * p.ldx) % 4);
                base = (const float *)p.X + c * p.ldx - delta;
            }
            tp.cls_rows[c] = rows_c;
            tp.cls_delta[c] = delta;
            u += (int)(ceil_div(rows_c, br) * p.splits);
            if (rows_c == 0) continue;
            okm = okm && (p.tx ? make_tmap_f32(&maps.x[c], base, (uint64_t)p.rows, (uint64_t)p.K,
                                               (uint64_t)p.ldx * 4, 256, thin::BK, false)
                               : make_tmap_f32(&maps.x[c], base, (uint64_t)(p.K + delta), (uint64_t)rows_c,
                                               (uint64_t)p.ldx * 4 * (classes ? 4 : 1), thin::BK, 256, true));
        }
        tp.cls_u0[4] = u;
        if (!okm) return set_status(GB_ERR_CUDA, "skinny: cuTensorMapEncodeTiled failed");
        int *err = error_word();
        if (!err) return set_status(GB_ERR_OOM, "skinny: no device error word");
        tp.C = p.C; tp.cs_r = p.cs_r; tp.cs_c = p.cs_c; tp.alpha = (float)p.alpha; tp.beta = (float)p.beta;
        tp.semantics = p.semantics; tp.part = (float *)p.part; tp.err = err;
        const int grid = u < sm_count() ? u : sm_count();
        if (grid == 0) return ok();
        gb_status s;
        const bool wt = p.tw && !pack;
        const int sel = (ns == 8 ? 4 : 0) | (p.tx ? 2 : 0) | (wt ? 1 : 0);
        switch (sel) {
            case 0: s = launch_thin<4, false, false>(maps, tp, grid, st); break;
            case 1: s = launch_thin<4, false, true>(maps, tp, grid, st); break;
            case 2: s = launch_thin<4, true, false>(maps, tp, grid, st); break;
            case 3: s = launch_thin<4, true, true>(maps, tp, grid, st); break;
            case 4: s = launch_thin<8, false, false>(maps, tp, grid, st); break;
            case 5: s = launch_thin<8, false, true>(maps, tp, grid, st); break;
            case 6: s = launch_thin<8, true, false>(maps, tp, grid, st); break;
            default: s = launch_thin<8, true, true>(maps, tp, grid, st); break;
        }
        if (s != GB_OK) return s;
        if (p.splits > 1) {
            int blocks = (int)(ceil_div(p.rows * p.n, 256) < 4 * sm_count() ? ceil_div(p.rows * p.n, 256)
                                                                             : 4 * sm_count());
            skinny_reduce_kernel<T, NB><<<blocks, 256, 0, st>>>(p);
            GB_LAUNCH_CHECK("skinny_reduce_kernel");
        }
        return ok();
    }
    dim3 grid((unsigned)pl.rtiles, (unsigned)p.splits);
    if (pl.rows_kernel) {
        if (pl.vec && pl.wvec) skinny_rows_kernel<T, NB, true, true><<<grid, NT, 0, st>>>(p);
        else if (pl.vec) skinny_rows_kernel<T, NB, true, false><<<grid, NT, 0, st>>>(p);
        else skinny_rows_kernel<T, NB, false, false><<<grid, NT, 0, st>>>(p);
    } else {
        if (pl.vec) skinny_cols_kernel<T, NB, true><<<grid, NT, 0, st>>>(p);
        else skinny_cols_kernel<T, NB, false><<<grid, NT, 0, st>>>(p);
    }
    GB_LAUNCH_CHECK("skinny kernel");
    if (p.splits > 1) {
        int blocks = (int)(ceil_div(p.rows * p.n, 256) < 4 * sm_count() ? ceil_div(p.rows * p.n, 256) : 4 * sm_count());
        skinny_reduce_kernel<T, NB><<<blocks, 256, 0, st>>>(p);
        GB_LAUNCH_CHECK("skinny_reduce_kernel");
    }
    return ok();
}

template <typename T, int NB>
gb_status run(SkParams p, cudaStream_t st) {
    Plan pl;
    gb_status s = make_plan<T, NB>(p, pl);
    if (s != GB_OK) return s;
    if (pl.part_bytes || pl.w_bytes) {
        // one workspace block: partials, then the W pieces (256-byte aligned)
        const size_t off = (pl.part_bytes + 255) / 256 * 256;
        uint8_t *ws = (uint8_t *)workspace(off + pl.w_bytes, st);
        if (!ws) return (gb_status)gb_get_last_status();
        p.part = pl.part_bytes ? ws : nullptr;
        p.wpieces = pl.w_bytes ? ws + off : nullptr;
    }
    return launch_plan<T, NB>(p, pl, st);
}

// X/W roles: thinB (N <= M) uses X = op(A), W = op(B); shortA the transpose.
void set_roles(SkParams &p, bool ta, bool tb, int64_t M, int64_t N, const void *A, int64_t lda, const void *B,
               int64_t ldb, int64_t ldc) {
    if (N <= M) {   // C (M x N) = op(A) op(B)
        p.rows = M; p.X = A; p.ldx = lda; p.tx = ta;
        p.W = B; p.ldw = ldb; p.tw = tb; p.n = (int)(N < 65 ? N : 65);
        p.cs_r = ldc; p.cs_c = 1;
    } else {        // C^T (N x M) = op(B)^T op(A)^T
        p.rows = N; p.X = B; p.ldx = ldb; p.tx = !tb;
        p.W = A; p.ldw = lda; p.tw = !ta; p.n = (int)(M < 65 ? M : 65);
        p.cs_r = 1; p.cs_c = ldc;
    }
}

// The workspace run<T, NB> takes for the plan of p (bytes; 0 when the plan fails).
template <typename T, int NB>
size_t plan_bytes(SkParams p) {
    Plan pl;
    if (make_plan<T, NB>(p, pl) != GB_OK) return 0;
    if (!pl.part_bytes && !pl.w_bytes) return 0;
    return (pl.part_bytes + 255) / 256 * 256 + pl.w_bytes;
}

// need == nullptr: run the product.  Otherwise: store the workspace the run
// would take in *need and launch nothing.
template <typename T>
gb_status dispatch(const GemmArgs &g, size_t *need = nullptr) {
    if (need) *need = 0;
    if (g.M == 0 || g.N == 0) return ok();
    SkParams p{};
    set_roles(p, g.ta, g.tb, g.M, g.N, g.A, g.lda, g.B, g.ldb, g.ldc);
    p.K = g.K; p.C = g.C; p.alpha = g.alpha; p.beta = g.beta; p.semantics = g.semantics;
    p.want_splits = g.split_k;
    if (p.n > 64) return set_status(GB_ERR_UNSUPPORTED, "skinny: small dimension %lld > 64",
                                    (long long)(g.M < g.N ? g.M : g.N));
    if (sizeof(T) == 8 && thin_oz_eligible(p.tx, p.ldx, p.X, p.rows, p.K)) {
        // FP64: digits on the tensor cores; units of 128 rows x K chunks of
        // 512, split K until there are ~4 units per SM
        const int64_t rtiles = ceil_div(p.rows, 128), nchunks = ceil_div(p.K, 512);
        int splits = 1;
        while (rtiles * splits < 4 * (int64_t)sm_count() && nchunks / (splits * 2) >= 2 && splits < 64) splits *= 2;
        if (g.split_k > 0) splits = g.split_k;
        const int64_t cpc = ceil_div(nchunks, splits);
        splits = (int)ceil_div(nchunks, cpc);
        if (need) {
            *need = thin_oz_workspace_bytes(p.rows, p.K, p.n, splits);
            return ok();
        }
        void *ws = workspace(thin_oz_workspace_bytes(p.rows, p.K, p.n, splits), g.stream);
        if (!ws) return (gb_status)gb_get_last_status();
        return launch_thin_oz(p.rows, p.K, (const double *)p.X, p.ldx, p.tx, (const double *)p.W, p.ldw, p.tw, p.n,
                              (double *)p.C, p.cs_r, p.cs_c, p.alpha, p.beta, p.semantics, splits, cpc * 512, ws,
                              g.stream);
    }
    if (need) {
        *need = p.n <= 8 ? plan_bytes<T, 8>(p) : p.n <= 16 ? plan_bytes<T, 16>(p)
              : p.n <= 32 ? plan_bytes<T, 32>(p) : plan_bytes<T, 64>(p);
        return ok();
    }
    if (p.n <= 8) return run<T, 8>(p, g.stream);
    if (p.n <= 16) return run<T, 16>(p, g.stream);
    if (p.n <= 32) return run<T, 32>(p, g.stream);
    return run<T, 64>(p, g.stream);
}

}  // namespace

gb_status launch_skinny_f32(const GemmArgs &g) { return dispatch<float>(g); }
gb_status launch_skinny_f64(const GemmArgs &g) { return dispatch<double>(g); }

size_t skinny_workspace_bytes(const GemmArgs &g, int bits) {
    size_t need = 0;
    const gb_status st = bits == 64 ? dispatch<double>(g, &need) : dispatch<float>(g, &need);
    return st == GB_OK ? need : 0;
}

}  // namespace gb

// ---------------------------------------------------------------------------
// gb_sgemm_skinny_noalloc: the FP32 skinny GEMM for callers that cannot
// allocate device memory on the call path.  It is the FFMA kernels with the
// same split-K plan as the GB_ALGO_SKINNY path above (for 8 < n <= 64 that
// path runs on the tensor cores instead, whose W pieces need scratch of
// their own, so here n > 8 keeps the FFMA streaming kernels), but the split-K
// partial sums live in a fixed array of device memory reserved when the
// library is loaded, so the call itself never calls cudaMalloc / cudaFree or
// any allocating routine.
#include <mutex>

namespace gb {
namespace {

// Size of the fixed split-K scratch.  Every GPU that loads the library keeps
// this array until the process exits.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;   // 16 MiB

static __device__ __align__(256) unsigned char g_skinny_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxNoAllocDev = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[kMaxNoAllocDev] = {nullptr};

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked
// up once per device (with that device current) and cached.
gb_status noalloc_scratch(void **out) {
    int dev = -1;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxNoAllocDev)
        return set_status(GB_ERR_UNSUPPORTED, "gb_sgemm_skinny_noalloc: device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_skinny_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) return cuda_status(e, "cudaGetSymbolAddress(skinny no-alloc scratch)");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return ok();
}

// The plan and kernels of run<float, NB>() with the static scratch in place
// of the library workspace.  Every partial the reduce kernel reads is
// written by the first kernel of the same call, so nothing has to be
// cleared between calls.
template <int NB>
gb_status run_noalloc(SkParams p, cudaStream_t st) {
    Plan pl;
    gb_status s = make_plan<float, NB>(p, pl, /*allow_tc=*/false);
    if (s != GB_OK) return s;
    if (pl.part_bytes || pl.w_bytes) {
        // partial sums first, then the packed W (256-byte aligned), as in run()
        const size_t off = (pl.part_bytes + 255) / 256 * 256;
        if (off + pl.w_bytes > kNoAllocScratchBytes)
            return set_status(GB_ERR_INVALID_ARG,
                              "gb_sgemm_skinny_noalloc: %d-way split-K over %lld rows needs %zu bytes of scratch, "
                              "more than the fixed %zu bytes",
                              p.splits, (long long)p.rows, off + pl.w_bytes, kNoAllocScratchBytes);
        void *base = nullptr;
        s = noalloc_scratch(&base);
        if (s != GB_OK) return s;
        p.part = pl.part_bytes ? base : nullptr;
        p.wpieces = pl.w_bytes ? (unsigned char *)base + off : nullptr;
    }
    return launch_plan<float, NB>(p, pl, st);
}

}  // namespace
}  // namespace gb

extern "C" gb_status gb_sgemm_skinny_noalloc(char transA, char transB, int64_t M, int64_t N, int64_t K, float alpha,
                                             const float *A, int64_t lda, const float *B, int64_t ldb, float beta,
                                             float *C, int64_t ldc, int semantics, void *stream) {
    using namespace gb;
    const char *fn = "gb_sgemm_skinny_noalloc";
    GB_CHECK_ARG(is_mode(transA) && is_mode(transB), "%s: transA/transB must be 'N' or 'T'", fn);
    GB_CHECK_ARG(M >= 0 && N >= 0 && K >= 0, "%s: negative dimension", fn);
    GB_CHECK_ARG(semantics >= 0 && semantics <= 2, "%s: unknown semantics %d", fn, semantics);
    const bool ta = is_trans(transA), tb = is_trans(transB);
    const int64_t acols = ta ? M : K, bcols = tb ? K : N;
    GB_CHECK_ARG(lda >= (acols > 1 ? acols : 1), "%s: lda (%lld) < %lld", fn, (long long)lda, (long long)acols);
    GB_CHECK_ARG(ldb >= (bcols > 1 ? bcols : 1), "%s: ldb (%lld) < %lld", fn, (long long)ldb, (long long)bcols);
    GB_CHECK_ARG(ldc >= (N > 1 ? N : 1), "%s: ldc (%lld) < N (%lld)", fn, (long long)ldc, (long long)N);
    if (M == 0 || N == 0) return ok();
    GB_CHECK_ARG(K > 0, "%s: K must be positive (K == 0 has no product to compute; use gb_sgemm)", fn);
    GB_CHECK_ARG(A && B && C, "%s: null pointer", fn);
    SkParams p{};
    set_roles(p, ta, tb, M, N, A, lda, B, ldb, ldc);
    GB_CHECK_ARG(p.n <= 64, "%s: min(M, N) must be <= 64 (got M=%lld, N=%lld)", fn, (long long)M, (long long)N);
    p.K = K; p.C = C; p.alpha = alpha; p.beta = beta; p.semantics = semantics;
    cudaStream_t st = as_stream(stream);
    if (p.n <= 8) return run_noalloc<8>(p, st);
    if (p.n <= 16) return run_noalloc<16>(p, st);
    if (p.n <= 32) return run_noalloc<32>(p, st);
    return run_noalloc<64>(p, st);
}
