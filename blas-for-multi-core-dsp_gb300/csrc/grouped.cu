// grouped.cu -- one persistent kernel over many independent GEMMs.
//
// A batch of GEMMs of uneven shapes, transpose modes, semantics and dtypes
// (FP32 and FP64 mixed) is described by a device work list; a persistent
// grid of CTAs pulls 64 x 64 C tiles from the whole list through one atomic
// counter, so small problems that could not fill the GPU alone share it.
// The reference runs one problem at a time per DSP cluster; this is the
// GB300 batching layer of the serving path and has no reference counterpart.
//
// The work list travels host -> device with one copy per batch from a pinned
// staging buffer; each staging slot owns its device list, an event guarding
// reuse, and (optionally) a CUDA graph of [copy, kernel] captured once and
// replayed for every batch that uses the slot.
#include <string.h>

#include <mutex>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace gb {
namespace {

constexpr int TM = 64, TN = 64, TK = 16, NT = 256;

struct alignas(16) GItem {
    const void *A, *B;
    void *C;
    int64_t M, N, K, lda, ldb, ldc;
    double alpha, beta;
    int32_t bits, ta, tb, semantics;
    int32_t tiles_n, tile_base;
};

struct alignas(16) GHeader {
    int32_t count, total_tiles, counter, pad;
};

template <typename T>
__device__ void tile_gemm(const GItem &g, int tm, int tn, unsigned char *smem) {
    T(*As)[TM + 1] = reinterpret_cast<T(*)[TM + 1]>(smem);
    T(*Bs)[TN + 1] = reinterpret_cast<T(*)[TN + 1]>(smem + sizeof(T) * TK * (TM + 1));
    const T *A = (const T *)g.A, *B = (const T *)g.B;
    T *C = (T *)g.C;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const int64_t m0 = (int64_t)tm * TM, n0 = (int64_t)tn * TN;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = T(0);
    for (int64_t k0 = 0; k0 < g.K; k0 += TK) {
        __syncthreads();
#pragma unroll
        for (int r = 0; r < (TM * TK) / NT; r++) {
            int l = tid + r * NT, mm, kk;
            if (g.ta) { mm = l % TM; kk = l / TM; } else { mm = l / TK; kk = l % TK; }
            int64_t m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < g.M && k < g.K) ? (g.ta ? A[k * g.lda + m] : A[m * g.lda + k]) : T(0);
        }
#pragma unroll
        for (int r = 0; r < (TN * TK) / NT; r++) {
            int l = tid + r * NT, nn, kk;
            if (g.tb) { nn = l / TK; kk = l % TK; } else { nn = l % TN; kk = l / TN; }
            int64_t n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < g.N && k < g.K) ? (g.tb ? B[n * g.ldb + k] : B[k * g.ldb + n]) : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; kk++) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int64_t m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
            if (m >= g.M || n >= g.N) continue;
            T *cp = C + m * g.ldc + n;
            T v = (T)g.alpha * acc[i][j];
            if (g.semantics == GB_SEM_BLAS) {
                if (g.beta != 0.0) v = fma((T)g.beta, *cp, v);
            } else if (g.semantics == GB_SEM_SCALAR_BETA) {
                v = v + (T)g.beta;
            } else {
                v = *cp + (v + (T)g.beta);
            }
            *cp = v;
        }
}

__global__ void __launch_bounds__(NT) grouped_gemm_kernel(GHeader *hdr, const GItem *items) {
    __shared__ __align__(16) unsigned char smem[2 * sizeof(double) * TK * (TM + 1)];
    __shared__ int s_tile;
    const int count = hdr->count, total = hdr->total_tiles;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_tile = atomicAdd(&hdr->counter, 1);
        __syncthreads();
        const int t = s_tile;
        if (t >= total) break;
        // item whose tile range holds t (tile_base is increasing)
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) / 2;
            if (items[mid].tile_base <= t) lo = mid; else hi = mid - 1;
        }
        const GItem g = items[lo];
        const int local = t - g.tile_base;
        const int tm = local / g.tiles_n, tn = local - tm * g.tiles_n;
        if (g.bits == 64) tile_gemm<double>(g, tm, tn, smem);
        else tile_gemm<float>(g, tm, tn, smem);
    }
}

// A pinned staging buffer + device work list + reuse event (+ graph).
struct Slot {
    unsigned char *host = nullptr;
    unsigned char *dev = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graph_stream = nullptr;
    int graph_grid = 0;
};

}  // namespace

struct GroupRunner {
    std::mutex mu;
    std::vector<Slot> slots;
    size_t next = 0;
    int max_items;

    explicit GroupRunner(int nslots, int max_items_) : slots(nslots), max_items(max_items_) {}

    ~GroupRunner() {
        for (auto &s : slots) {
            if (s.done) cudaEventSynchronize(s.done);
            if (s.graph) cudaGraphExecDestroy(s.graph);
            if (s.done) cudaEventDestroy(s.done);
            if (s.host) cudaFreeHost(s.host);
            if (s.dev) cudaFree(s.dev);
        }
    }

    gb_status prepare(Slot &s) {
        const size_t need = sizeof(GHeader) + sizeof(GItem) * (size_t)max_items;
        if (s.cap >= need) return ok();
        GB_CUDA_TRY(cudaHostAlloc((void **)&s.host, need, cudaHostAllocDefault));
        GB_CUDA_TRY(cudaMalloc((void **)&s.dev, need));
        GB_CUDA_TRY(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
        s.cap = need;
        return ok();
    }

    // Build the work list for n descriptors; launch on `stream`.
    gb_status run(const gb_gemm_desc *d, int n, cudaStream_t stream, bool use_graph) {
        if (n > max_items) return set_status(GB_ERR_INVALID_ARG, "gb_gemm_batch: %d GEMMs > capacity %d", n, max_items);
        Slot *sp;
        {
            std::lock_guard<std::mutex> lk(mu);
            sp = &slots[next];
            next = (next + 1) % slots.size();
        }
        Slot &s = *sp;
        gb_status st = prepare(s);
        if (st != GB_OK) return st;
        GB_CUDA_TRY(cudaEventSynchronize(s.done));   // previous batch in this slot finished reading it
        GHeader *h = reinterpret_cast<GHeader *>(s.host);
        GItem *it = reinterpret_cast<GItem *>(s.host + sizeof(GHeader));
        int tiles = 0, count = 0;
        for (int i = 0; i < n; i++) {
            const gb_gemm_desc &q = d[i];
            if (q.M == 0 || q.N == 0) continue;
            GItem &g = it[count++];
            g.A = q.A; g.B = q.B; g.C = q.C;
            g.M = q.M; g.N = q.N; g.K = q.K; g.lda = q.lda; g.ldb = q.ldb; g.ldc = q.ldc;
            g.alpha = q.alpha; g.beta = q.beta;
            g.bits = q.dtype_bits; g.ta = is_trans(q.transA); g.tb = is_trans(q.transB); g.semantics = q.semantics;
            g.tiles_n = (int)ceil_div(q.N, TN);
            g.tile_base = tiles;
            tiles += (int)(ceil_div(q.M, TM) * g.tiles_n);
        }
        h->count = count;
        h->total_tiles = tiles;
        h->counter = 0;
        h->pad = 0;
        if (count == 0) return ok();
        const size_t bytes = sizeof(GHeader) + sizeof(GItem) * (size_t)max_items;
        const int grid = 2 * sm_count();
        if (use_graph) {
            if (!s.graph || s.graph_stream != stream) {
                if (s.graph) cudaGraphExecDestroy(s.graph);
                s.graph = nullptr;
                cudaStream_t cap;
                GB_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
                cudaGraph_t gr;
                cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
                cudaMemcpyAsync(s.dev, s.host, bytes, cudaMemcpyHostToDevice, cap);
                grouped_gemm_kernel<<<grid, NT, 0, cap>>>(reinterpret_cast<GHeader *>(s.dev),
                                                          reinterpret_cast<const GItem *>(s.dev + sizeof(GHeader)));
                cudaError_t e = cudaStreamEndCapture(cap, &gr);
                cudaStreamDestroy(cap);
                if (e != cudaSuccess) return cuda_status(e, "grouped graph capture");
                e = cudaGraphInstantiate(&s.graph, gr, 0);
                cudaGraphDestroy(gr);
                if (e != cudaSuccess) return cuda_status(e, "grouped graph instantiate");
                s.graph_stream = stream;
                s.graph_grid = grid;
            }
            count_launch();
            GB_CUDA_TRY(cudaGraphLaunch(s.graph, stream));
        } else {
            GB_CUDA_TRY(cudaMemcpyAsync(s.dev, s.host, bytes, cudaMemcpyHostToDevice, stream));
            grouped_gemm_kernel<<<grid, NT, 0, stream>>>(reinterpret_cast<GHeader *>(s.dev),
                                                         reinterpret_cast<const GItem *>(s.dev + sizeof(GHeader)));
            GB_LAUNCH_CHECK("grouped_gemm_kernel");
        }
        GB_CUDA_TRY(cudaEventRecord(s.done, stream));
        return ok();
    }
};

GroupRunner *group_runner_create(int nslots, int max_items) { return new GroupRunner(nslots, max_items); }
void group_runner_destroy(GroupRunner *r) { delete r; }
gb_status group_runner_run(GroupRunner *r, const gb_gemm_desc *d, int n, void *stream, int use_graph) {
    return r->run(d, n, as_stream(stream), use_graph != 0);
}

gb_status check_desc(const gb_gemm_desc &q, int i) {
    GB_CHECK_ARG(q.dtype_bits == 32 || q.dtype_bits == 64, "gemm %d: dtype_bits must be 32 or 64", i);
    GB_CHECK_ARG(is_mode(q.transA) && is_mode(q.transB), "gemm %d: transA/transB must be 'N' or 'T'", i);
    GB_CHECK_ARG(q.M >= 0 && q.N >= 0 && q.K >= 0, "gemm %d: negative dimension", i);
    GB_CHECK_ARG(q.semantics >= 0 && q.semantics <= 2, "gemm %d: unknown semantics", i);
    const int64_t acols = is_trans(q.transA) ? q.M : q.K, bcols = is_trans(q.transB) ? q.K : q.N;
    GB_CHECK_ARG(q.lda >= (acols > 1 ? acols : 1) && q.ldb >= (bcols > 1 ? bcols : 1) && q.ldc >= (q.N > 1 ? q.N : 1),
                 "gemm %d: leading dimension too small", i);
    if (q.M > 0 && q.N > 0) {
        GB_CHECK_ARG(q.C != nullptr, "gemm %d: C is null", i);
        if (q.K > 0) GB_CHECK_ARG(q.A && q.B, "gemm %d: A or B is null", i);
    }
    GB_CHECK_ARG(ceil_div(q.M, TM) * ceil_div(q.N, TN) < (1ll << 30), "gemm %d: too many tiles", i);
    return ok();
}

}  // namespace gb

static std::mutex g_batch_mu;
static gb::GroupRunner *g_batch_runner = nullptr;

extern "C" gb_status gb_gemm_batch(const gb_gemm_desc *descs, int n, void *stream) {
    using namespace gb;
    GB_CHECK_ARG(n >= 0, "gb_gemm_batch: negative count");
    if (n == 0) return ok();
    GB_CHECK_ARG(descs != nullptr, "gb_gemm_batch: null descriptor array");
    GB_CHECK_ARG(n <= 4096, "gb_gemm_batch: at most 4096 GEMMs per batch");
    int64_t tiles = 0;
    for (int i = 0; i < n; i++) {
        gb_status st = check_desc(descs[i], i);
        if (st != GB_OK) return st;
        tiles += ceil_div(descs[i].M, 64) * ceil_div(descs[i].N, 64);
    }
    GB_CHECK_ARG(tiles < (1ll << 30), "gb_gemm_batch: too many tiles in one batch");
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (!g_batch_runner) g_batch_runner = group_runner_create(4, 4096);
    return group_runner_run(g_batch_runner, descs, n, stream, 0);
}

// Strided batch: GEMM i uses A + i*strideA, B + i*strideB, C + i*strideC
// (strides in elements), all with the same shape, modes and scalars; run as
// grouped launches of up to 4096 GEMMs.
extern "C" gb_status gb_gemm_strided_batched(int dtype_bits, char transA, char transB, int64_t M, int64_t N,
                                             int64_t K, double alpha, const void *A, int64_t lda, int64_t strideA,
                                             const void *B, int64_t ldb, int64_t strideB, double beta, void *C,
                                             int64_t ldc, int64_t strideC, int64_t batch, int semantics,
                                             void *stream) {
    using namespace gb;
    GB_CHECK_ARG(dtype_bits == 32 || dtype_bits == 64, "gb_gemm_strided_batched: dtype_bits must be 32 or 64");
    GB_CHECK_ARG(batch >= 0, "gb_gemm_strided_batched: negative batch count");
    GB_CHECK_ARG(strideA >= 0 && strideB >= 0 && strideC >= 0, "gb_gemm_strided_batched: negative stride");
    if (batch == 0) return ok();
    // distinct C matrices must not overlap: strideC covers one C (rows x ldc)
    GB_CHECK_ARG(batch == 1 || strideC >= (M > 0 ? (M - 1) * ldc + N : 0),
                 "gb_gemm_strided_batched: strideC %lld smaller than one C", (long long)strideC);
    const size_t es = dtype_bits / 8;
    std::vector<gb_gemm_desc> d((size_t)(batch < 4096 ? batch : 4096));
    for (int64_t b0 = 0; b0 < batch; b0 += 4096) {
        const int n = (int)(batch - b0 < 4096 ? batch - b0 : 4096);
        for (int i = 0; i < n; i++) {
            gb_gemm_desc &q = d[i];
            memset(&q, 0, sizeof(q));
            q.dtype_bits = dtype_bits; q.transA = transA; q.transB = transB; q.semantics = semantics;
            q.M = M; q.N = N; q.K = K; q.alpha = alpha; q.beta = beta;
            q.A = (const char *)A + (size_t)(b0 + i) * strideA * es; q.lda = lda;
            q.B = (const char *)B + (size_t)(b0 + i) * strideB * es; q.ldb = ldb;
            q.C = (char *)C + (size_t)(b0 + i) * strideC * es; q.ldc = ldc;
        }
        gb_status st = gb_gemm_batch(d.data(), n, stream);
        if (st != GB_OK) return st;
    }
    return ok();
}
