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
//    16-byte loads (lane l holds k = 32*V*step + V*l .. +V-1), multiplies by
//    the W slab kept lane-contiguous in shared memory (conflict-free), and
//    reduces across lanes with shuffles at the end.
//  * X K-major (rows contiguous): each thread owns R rows, loads are
//    coalesced across lanes, W is read by broadcast from shared memory.
// Split-K over CTAs when the row count alone cannot fill the GPU; partial
// sums go to scratch and a second kernel applies alpha/beta.
#include "gb_common.cuh"

namespace gb {
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
    void *part;                           // splits x rows x NB partials (split-K only)
};

// row-major X: R rows per warp, W slab of SLAB k's (<= 32 KB of shared memory)
template <typename T, int NB>
struct RowCfg {
    static constexpr int V = 16 / (int)sizeof(T);   // elements per 16-byte load
    static constexpr int KS = 32 * V;               // k per warp step
    static constexpr int R = NB <= 8 ? 8 : NB <= 16 ? 4 : NB <= 32 ? 2 : 1;
    static constexpr int STEPS = (32768 / (int)sizeof(T) / NB) / KS;
    static constexpr int SLAB = STEPS * KS;
    static constexpr int BR = (NT / 32) * R;        // rows per CTA
};

// K-major X: R rows per thread
template <typename T, int NB>
struct ColCfg {
    static constexpr int R = NB <= 16 ? 4 : NB <= 32 ? 2 : 1;
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

template <typename T, int NB, bool VEC>
__global__ void __launch_bounds__(NT) skinny_rows_kernel(SkParams p) {
    using C = RowCfg<T, NB>;
    constexpr int V = C::V, KS = C::KS, R = C::R;
    __shared__ __align__(16) T Ws[C::SLAB * NB];   // [step][q][j][lane]
    const T *X = (const T *)p.X;
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

    for (int64_t k0 = kbeg; k0 < kend; k0 += C::SLAB) {
        const int cnt = (int)((kend - k0) < C::SLAB ? (kend - k0) : C::SLAB);
        __syncthreads();
        // Ws[((s*V + q)*NB + j)*32 + l] holds W(k0 + s*KS + l*V + q, j)
        stage_w<T, NB>(p, Ws, k0, C::SLAB, kend, [](int e, int &kk, int &j) {
            const int l = e % 32, r1 = e / 32;
            j = r1 % NB;
            const int r2 = r1 / NB, q = r2 % V, st = r2 / V;
            kk = st * KS + l * V + q;
        });
        __syncthreads();
        const int steps = (cnt + KS - 1) / KS;
        for (int s = 0; s < steps; s++) {
            const int64_t kb = k0 + (int64_t)s * KS + lane * V;
            T xv[R][V];
#pragma unroll
            for (int i = 0; i < R; i++) {
                const int64_t row = r0 + i;
                const T *xp = X + row * p.ldx + kb;
                if (VEC && row < p.rows && kb + V <= kend) {
                    if (sizeof(T) == 4) {
                        float4 v = __ldg(reinterpret_cast<const float4 *>(xp));
                        reinterpret_cast<float *>(xv[i])[0] = v.x;
                        reinterpret_cast<float *>(xv[i])[1] = v.y;
                        reinterpret_cast<float *>(xv[i])[2] = v.z;
                        reinterpret_cast<float *>(xv[i])[3] = v.w;
                    } else {
                        double2 v = __ldg(reinterpret_cast<const double2 *>(xp));
                        reinterpret_cast<double *>(xv[i])[0] = v.x;
                        reinterpret_cast<double *>(xv[i])[1] = v.y;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < V; q++) xv[i][q] = (row < p.rows && kb + q < kend) ? xp[q] : T(0);
                }
            }
#pragma unroll
            for (int q = 0; q < V; q++)
#pragma unroll
                for (int j = 0; j < NB; j++) {
                    const T w = Ws[((s * V + q) * NB + j) * 32 + lane];
#pragma unroll
                    for (int i = 0; i < R; i++) acc[i][j] = fma(xv[i][q], w, acc[i][j]);
                }
        }
    }

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

template <typename T, int NB>
__global__ void __launch_bounds__(NT) skinny_cols_kernel(SkParams p) {
    using C = ColCfg<T, NB>;
    constexpr int R = C::R, U = C::U;
    __shared__ __align__(16) T Ws[C::SLAB * NB];   // [k][j]
    const T *X = (const T *)p.X;
    const int tid = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * C::BR;
    const int split = blockIdx.y;
    const int64_t kbeg = (int64_t)split * p.kchunk;
    const int64_t kend = kbeg + p.kchunk < p.K ? kbeg + p.kchunk : p.K;

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
                for (int i = 0; i < R; i++) {
                    const int64_t row = r0 + tid + i * NT;
                    x[u][i] = (kk + u < cnt && row < p.rows) ? __ldg(X + (k0 + kk + u) * p.ldx + row) : T(0);
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
    for (int i = 0; i < R; i++) {
        const int64_t row = r0 + tid + i * NT;
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
    bool rows_kernel, vec;
    int64_t rtiles;
    size_t part_bytes;
};

template <typename T, int NB>
gb_status make_plan(SkParams &p, Plan &pl) {
    pl.rows_kernel = !p.tx;
    const int64_t br = pl.rows_kernel ? RowCfg<T, NB>::BR : ColCfg<T, NB>::BR;
    const int64_t gran = pl.rows_kernel ? RowCfg<T, NB>::KS : 32;
    pl.rtiles = ceil_div(p.rows, br);
    if (pl.rtiles > 0x7fffffff) return set_status(GB_ERR_UNSUPPORTED, "skinny: too many rows");
    // split K until the grid covers ~2 waves of the GPU
    const int64_t target = 2 * (int64_t)sm_count();
    int splits = 1;
    while (pl.rtiles * splits < target && p.K / (splits * 2) >= 256 && splits < 64) splits *= 2;
    p.kchunk = ceil_div(ceil_div(p.K, splits), gran) * gran;
    p.splits = (int)ceil_div(p.K, p.kchunk);
    if (p.splits < 1) p.splits = 1;
    constexpr int V = RowCfg<T, NB>::V;
    pl.vec = pl.rows_kernel && (p.ldx % V == 0) && ((uintptr_t)p.X % 16 == 0);
    pl.part_bytes = p.splits > 1 ? (size_t)p.splits * p.rows * NB * sizeof(T) : 0;
    return ok();
}

template <typename T, int NB>
gb_status launch_plan(const SkParams &p, const Plan &pl, cudaStream_t st) {
    dim3 grid((unsigned)pl.rtiles, (unsigned)p.splits);
    if (pl.rows_kernel) {
        if (pl.vec) skinny_rows_kernel<T, NB, true><<<grid, NT, 0, st>>>(p);
        else skinny_rows_kernel<T, NB, false><<<grid, NT, 0, st>>>(p);
    } else {
        skinny_cols_kernel<T, NB><<<grid, NT, 0, st>>>(p);
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
    if (pl.part_bytes) {
        p.part = workspace(pl.part_bytes, st);
        if (!p.part) return (gb_status)gb_get_last_status();
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

template <typename T>
gb_status dispatch(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    SkParams p{};
    set_roles(p, g.ta, g.tb, g.M, g.N, g.A, g.lda, g.B, g.ldb, g.ldc);
    p.K = g.K; p.C = g.C; p.alpha = g.alpha; p.beta = g.beta; p.semantics = g.semantics;
    if (p.n > 64) return set_status(GB_ERR_UNSUPPORTED, "skinny: small dimension %lld > 64",
                                    (long long)(g.M < g.N ? g.M : g.N));
    if (p.n <= 8) return run<T, 8>(p, g.stream);
    if (p.n <= 16) return run<T, 16>(p, g.stream);
    if (p.n <= 32) return run<T, 32>(p, g.stream);
    return run<T, 64>(p, g.stream);
}

}  // namespace

gb_status launch_skinny_f32(const GemmArgs &g) { return dispatch<float>(g); }
gb_status launch_skinny_f64(const GemmArgs &g) { return dispatch<double>(g); }

}  // namespace gb

// ---------------------------------------------------------------------------
// gb_sgemm_skinny_noalloc: the FP32 skinny GEMM for callers that cannot
// allocate device memory on the call path.  It is the same kernels with the
// same split-K plan as the GB_ALGO_SKINNY path above, but the split-K
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
    gb_status s = make_plan<float, NB>(p, pl);
    if (s != GB_OK) return s;
    if (pl.part_bytes) {
        if (pl.part_bytes > kNoAllocScratchBytes)
            return set_status(GB_ERR_INVALID_ARG,
                              "gb_sgemm_skinny_noalloc: %d-way split-K over %lld rows needs %zu bytes of scratch, "
                              "more than the fixed %zu bytes",
                              p.splits, (long long)p.rows, pl.part_bytes, kNoAllocScratchBytes);
        s = noalloc_scratch(&p.part);
        if (s != GB_OK) return s;
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
