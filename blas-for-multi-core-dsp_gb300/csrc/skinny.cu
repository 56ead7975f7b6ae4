// skinny.cu -- bandwidth-bound GEMM for a tiny N (thinB) or a tiny M (shortA).
//
// Replaces irr_thinB_{s,d}gemm_{NN,NT,TN,TT}
// (irr_thinB_sgemm_release_V1.2/device_code/irr_thinB_sgemm_kernel.c:2910,
// 3448, 4619, 5147; irr_thinB_dgemm_release_V0.0/.../irr_thinB_dgemm_kernel.c:
// 1607, 1903, 2587, 2869) and irr_shortA_{s,d}gemm_* (irr_shortA_sgemm_kernel.c:
// 1769, 2034, 2592, 2820; irr_shortA_dgemm_kernel.c:1607, 1849, 2431, 2665).
//
// Like the reference, shortA is computed as the transpose of a thinB problem
// (C^T = op(B)^T op(A)^T), so one kernel streams the large operand ("X",
// rows x K) exactly once while the small one ("W", K x nb) is staged per K
// chunk in shared memory and read from L2 by every CTA.  The output is
// written through two strides, so C^T is never formed.
//
// CTA: 256 threads, each owning R consecutive-in-lane rows and all nb
// columns in registers (R*nb <= 64); the X tile is loaded along its
// contiguous dimension (k for a row-major X, rows for a transposed one) and
// stored K-major in shared memory.  Split-K over CTAs when the row count
// alone cannot fill the GPU; partial sums go to the library workspace and a
// second kernel applies alpha/beta.
#include "gb_common.cuh"

namespace gb {
namespace {

constexpr int NT = 256;
// K chunk staged per step: 32 KB of X tile in shared memory
template <typename T, int R>
struct SkTile { static constexpr int BK = (32768 / (int)sizeof(T)) / (NT * R); };

struct SkParams {
    int64_t rows, K;            // X is rows x K (logical)
    const void *X; int64_t ldx; int tx;   // tx: X stored transposed (K x rows)
    const void *W; int64_t ldw; int tw;   // W logical K x n; tw: stored n x K
    int n;                      // logical small dimension (<= nb)
    void *C; int64_t cs_r, cs_c;  // C(r, j) at C[r*cs_r + j*cs_c]
    double alpha, beta;
    int semantics;
    int splits; int64_t kchunk;  // split-K
    void *part;                 // splits x rows x nb partials (split-K only)
};

template <typename T, int NB, int R>
__global__ void __launch_bounds__(NT) skinny_kernel(SkParams p) {
    constexpr int BR = NT * R;            // rows per CTA
    constexpr int BK = SkTile<T, R>::BK;
    __shared__ __align__(16) T Xs[BK][BR];
    __shared__ __align__(16) T Ws[BK][NB];
    const T *X = (const T *)p.X;
    const T *W = (const T *)p.W;
    const int tid = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * BR;
    const int split = blockIdx.y;
    const int64_t kbeg = (int64_t)split * p.kchunk;
    const int64_t kend = kbeg + p.kchunk < p.K ? kbeg + p.kchunk : p.K;

    T acc[R][NB];
#pragma unroll
    for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < NB; j++) acc[i][j] = T(0);

    for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
        __syncthreads();
        // X tile: BR rows x BK k's
        if (!p.tx) {
            // row-major X (rows x K): a warp reads BK consecutive k of one row
            for (int l = tid; l < BR * BK; l += NT) {
                int rr = l / BK, kk = l % BK;
                int64_t r = r0 + rr, k = k0 + kk;
                Xs[kk][rr] = (r < p.rows && k < kend) ? X[r * p.ldx + k] : T(0);
            }
        } else {
            // X stored K x rows: consecutive threads read consecutive rows
            for (int l = tid; l < BR * BK; l += NT) {
                int kk = l / BR, rr = l % BR;
                int64_t r = r0 + rr, k = k0 + kk;
                Xs[kk][rr] = (r < p.rows && k < kend) ? X[k * p.ldx + r] : T(0);
            }
        }
        for (int l = tid; l < BK * NB; l += NT) {
            int kk = l / NB, j = l % NB;
            int64_t k = k0 + kk;
            T v = T(0);
            if (j < p.n && k < kend) v = p.tw ? W[(int64_t)j * p.ldw + k] : W[k * p.ldw + j];
            Ws[kk][j] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < BK; kk++) {
            T x[R];
#pragma unroll
            for (int i = 0; i < R; i++) x[i] = Xs[kk][tid + i * NT];
#pragma unroll
            for (int j = 0; j < NB; j++) {
                T w = Ws[kk][j];
#pragma unroll
                for (int i = 0; i < R; i++) acc[i][j] = fma(x[i], w, acc[i][j]);
            }
        }
    }

#pragma unroll
    for (int i = 0; i < R; i++) {
        int64_t r = r0 + tid + i * NT;
        if (r >= p.rows) continue;
        if (p.splits > 1) {
            T *part = (T *)p.part + ((int64_t)split * p.rows + r) * NB;
#pragma unroll
            for (int j = 0; j < NB; j++) part[j] = acc[i][j];
            continue;
        }
#pragma unroll
        for (int j = 0; j < NB; j++) {
            if (j >= p.n) break;
            T *cp = (T *)p.C + r * p.cs_r + (int64_t)j * p.cs_c;
            T v = (T)p.alpha * acc[i][j];
            if (p.semantics == GB_SEM_BLAS) {
                if (p.beta != 0.0) v = fma((T)p.beta, *cp, v);
            } else if (p.semantics == GB_SEM_SCALAR_BETA) {
                v = v + (T)p.beta;
            } else {
                v = *cp + (v + (T)p.beta);
            }
            *cp = v;
        }
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
        T *cp = (T *)p.C + r * p.cs_r + (int64_t)j * p.cs_c;
        T v = (T)p.alpha * s;
        if (p.semantics == GB_SEM_BLAS) {
            if (p.beta != 0.0) v = fma((T)p.beta, *cp, v);
        } else if (p.semantics == GB_SEM_SCALAR_BETA) {
            v = v + (T)p.beta;
        } else {
            v = *cp + (v + (T)p.beta);
        }
        *cp = v;
    }
}

template <typename T, int NB, int R>
gb_status run(SkParams p, cudaStream_t st) {
    constexpr int BR = NT * R;
    const int64_t rtiles = ceil_div(p.rows, BR);
    if (rtiles > 0x7fffffff) return set_status(GB_ERR_UNSUPPORTED, "skinny: too many rows");
    // split K until the grid covers ~2 waves of the GPU
    const int64_t target = 2 * (int64_t)sm_count();
    int splits = 1;
    while (rtiles * splits < target && p.K / (splits * 2) >= 256 && splits < 64) splits *= 2;
    p.splits = splits;
    constexpr int BK = SkTile<T, R>::BK;
    p.kchunk = ceil_div(ceil_div(p.K, splits), BK) * BK;
    p.splits = (int)ceil_div(p.K, p.kchunk);
    if (p.splits < 1) p.splits = 1;
    if (p.splits > 1) {
        size_t bytes = (size_t)p.splits * p.rows * NB * sizeof(T);
        p.part = workspace(bytes, st);
        if (!p.part) return (gb_status)gb_get_last_status();
    }
    dim3 grid((unsigned)rtiles, (unsigned)p.splits);
    skinny_kernel<T, NB, R><<<grid, NT, 0, st>>>(p);
    GB_LAUNCH_CHECK("skinny_kernel");
    if (p.splits > 1) {
        int blocks = (int)(ceil_div(p.rows * p.n, 256) < 4 * sm_count() ? ceil_div(p.rows * p.n, 256) : 4 * sm_count());
        skinny_reduce_kernel<T, NB><<<blocks, 256, 0, st>>>(p);
        GB_LAUNCH_CHECK("skinny_reduce_kernel");
    }
    return ok();
}

template <typename T>
gb_status dispatch(const GemmArgs &g) {
    if (g.M == 0 || g.N == 0) return ok();
    SkParams p{};
    const bool thinB = g.N <= g.M;
    if (thinB) {   // C (M x N) = op(A) op(B): X = op(A), W = op(B)
        p.rows = g.M; p.X = g.A; p.ldx = g.lda; p.tx = g.ta;
        p.W = g.B; p.ldw = g.ldb; p.tw = g.tb; p.n = (int)g.N;
        p.cs_r = g.ldc; p.cs_c = 1;
    } else {       // C^T (N x M) = op(B)^T op(A)^T: X = op(B)^T, W = op(A)^T
        p.rows = g.N; p.X = g.B; p.ldx = g.ldb; p.tx = !g.tb;
        p.W = g.A; p.ldw = g.lda; p.tw = !g.ta; p.n = (int)g.M;
        p.cs_r = 1; p.cs_c = g.ldc;
    }
    p.K = g.K; p.C = g.C; p.alpha = g.alpha; p.beta = g.beta; p.semantics = g.semantics;
    if (p.n > 64) return set_status(GB_ERR_UNSUPPORTED, "skinny: small dimension %d > 64", p.n);
    if (p.n <= 8) return run<T, 8, 4>(p, g.stream);
    if (p.n <= 16) return run<T, 16, 4>(p, g.stream);
    if (p.n <= 32) return run<T, 32, 2>(p, g.stream);
    return run<T, 64, 1>(p, g.stream);
}

}  // namespace

gb_status launch_skinny_f32(const GemmArgs &g) { return dispatch<float>(g); }
gb_status launch_skinny_f64(const GemmArgs &g) { return dispatch<double>(g); }

}  // namespace gb

// ---------------------------------------------------------------------------
// gb_sgemm_skinny_noalloc: the FP32 skinny GEMM for callers that cannot
// allocate device memory on the call path.  It is the same two kernels with
// the same split-K plan as the GB_ALGO_SKINNY path above, but the split-K
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

// Mirrors run<float, NB, R>() above with the static scratch in place of the
// library workspace.  Every partial the reduce kernel reads is written by the
// first kernel of the same call, so nothing has to be cleared between calls.
template <int NB, int R>
gb_status run_noalloc(SkParams p, cudaStream_t st) {
    constexpr int BR = NT * R;
    const int64_t rtiles = ceil_div(p.rows, BR);
    if (rtiles > 0x7fffffff) return set_status(GB_ERR_UNSUPPORTED, "gb_sgemm_skinny_noalloc: too many rows");
    const int64_t target = 2 * (int64_t)sm_count();
    int splits = 1;
    while (rtiles * splits < target && p.K / (splits * 2) >= 256 && splits < 64) splits *= 2;
    constexpr int BK = SkTile<float, R>::BK;
    p.kchunk = ceil_div(ceil_div(p.K, splits), BK) * BK;
    p.splits = (int)ceil_div(p.K, p.kchunk);
    if (p.splits < 1) p.splits = 1;
    if (p.splits > 1) {
        const size_t bytes = (size_t)p.splits * p.rows * NB * sizeof(float);
        if (bytes > kNoAllocScratchBytes)
            return set_status(GB_ERR_INVALID_ARG,
                              "gb_sgemm_skinny_noalloc: %d-way split-K over %lld rows needs %zu bytes of scratch, "
                              "more than the fixed %zu bytes",
                              p.splits, (long long)p.rows, bytes, kNoAllocScratchBytes);
        void *s = nullptr;
        gb_status stt = noalloc_scratch(&s);
        if (stt != GB_OK) return stt;
        p.part = s;
    }
    dim3 grid((unsigned)rtiles, (unsigned)p.splits);
    skinny_kernel<float, NB, R><<<grid, NT, 0, st>>>(p);
    GB_LAUNCH_CHECK("skinny_kernel (no-alloc)");
    if (p.splits > 1) {
        int blocks = (int)(ceil_div(p.rows * p.n, 256) < 4 * sm_count() ? ceil_div(p.rows * p.n, 256) : 4 * sm_count());
        skinny_reduce_kernel<float, NB><<<blocks, 256, 0, st>>>(p);
        GB_LAUNCH_CHECK("skinny_reduce_kernel (no-alloc)");
    }
    return ok();
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
    if (N <= M) {
        p.rows = M; p.X = A; p.ldx = lda; p.tx = ta;
        p.W = B; p.ldw = ldb; p.tw = tb; p.n = (int)(N < 65 ? N : 65);
        p.cs_r = ldc; p.cs_c = 1;
    } else {
        p.rows = N; p.X = B; p.ldx = ldb; p.tx = !tb;
        p.W = A; p.ldw = lda; p.tw = !ta; p.n = (int)(M < 65 ? M : 65);
        p.cs_r = 1; p.cs_c = ldc;
    }
    GB_CHECK_ARG(p.n <= 64, "%s: min(M, N) must be <= 64 (got M=%lld, N=%lld)", fn, (long long)M, (long long)N);
    p.K = K; p.C = C; p.alpha = alpha; p.beta = beta; p.semantics = semantics;
    cudaStream_t st = as_stream(stream);
    if (p.n <= 8) return run_noalloc<8, 4>(p, st);
    if (p.n <= 16) return run_noalloc<16, 4>(p, st);
    if (p.n <= 32) return run_noalloc<32, 2>(p, st);
    return run_noalloc<64, 1>(p, st);
}
