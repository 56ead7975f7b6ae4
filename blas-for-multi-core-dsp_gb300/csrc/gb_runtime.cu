// gb_runtime.cu -- status codes, device queries, library workspace, memory
// helpers and the seeded input generator.
//
// Replaces the parts of the MT-3000 host runtime the reference's host demos
// use (hthread_dev_open / hthread_malloc / hthread_free,
// sgemm_release_V1.3.2/host_code/sgemm_demo.c:50-61, :338-351) with plain
// CUDA runtime calls.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "gb_common.cuh"
#include "sm100_ptx.cuh"

namespace gb {

static thread_local int t_status = GB_OK;
static thread_local char t_msg[512] = "";

gb_status set_status(gb_status st, const char *fmt, ...) {
    t_status = st;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
    va_end(ap);
    return st;
}

gb_status ok() { return GB_OK; }

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

gb_status cuda_status(cudaError_t e, const char *where) {
    return set_status(GB_ERR_CUDA, "%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
}

static const int kMaxDev = 64;

// A cap on the SMs this host thread's launches plan for (0: none): the persistent kernels size
// their grids from sm_count(), so a capped call leaves the other SMs to other streams' work.
static thread_local int t_sm_cap = 0;
void set_sm_cap(int cap) { t_sm_cap = cap > 0 ? cap : 0; }

int sm_count() {
    static int cache[kMaxDev] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDev) return 148;
    if (cache[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = n > 0 ? n : 148;
    }
    return t_sm_cap > 0 && t_sm_cap < cache[dev] ? t_sm_cap : cache[dev];
}

static uint64_t device_bit() {
    int dev = 0;
    cudaGetDevice(&dev);
    return 1ull << (dev & 63);
}

bool device_setup_needed(const std::atomic<uint64_t> &done) {
    return (done.load(std::memory_order_acquire) & device_bit()) == 0;
}

void device_setup_done(std::atomic<uint64_t> &done) { done.fetch_or(device_bit(), std::memory_order_acq_rel); }

int smem_optin() {
    static int cache[kMaxDev] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDev) return 227 * 1024;
    if (cache[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cache[dev] = n > 0 ? n : 227 * 1024;
    }
    return cache[dev];
}

static std::mutex g_ws_mu;
// one grow-only buffer per (device, stream): work queued on different
// streams never shares scratch
struct WsEntry {
    int dev;
    void *stream;
    void *ptr;
    size_t size;
    unsigned seq;   // calls that asked for a sequence number (workspace halves by parity)
};
static std::vector<WsEntry> g_ws;

void *workspace(size_t bytes, void *stream, unsigned *seq, size_t *size) {
    void *p = workspace(bytes, stream);
    if (p) {
        int dev = 0;
        cudaGetDevice(&dev);
        std::lock_guard<std::mutex> lk(g_ws_mu);
        for (auto &e : g_ws)
            if (e.dev == dev && e.stream == stream) {
                *seq = e.seq++;
                *size = e.size;
            }
    }
    return p;
}

// The (device, stream) entry of `pool`, grown to at least `bytes` (never below
// `floor`; a new buffer is cleared on the stream when `zero`).  Growing
// synchronises the stream (the old buffer may still be read by work queued on
// it) and is refused while the stream is being captured.
static void *pool_buffer(std::vector<WsEntry> &pool, size_t bytes, void *stream, size_t floor, const char *what,
                         bool zero = false, size_t *size = nullptr) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_ws_mu);
    WsEntry *w = nullptr;
    for (auto &e : pool)
        if (e.dev == dev && e.stream == stream) w = &e;
    if (w && w->size >= bytes) {
        if (size) *size = w->size;
        return w->ptr;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(as_stream(stream), &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone) {
        // growing would synchronise and free under the capture: the caller reserves first
        set_status(GB_ERR_INVALID_ARG, "%s: %zu bytes not reserved before the stream capture began (%zu held)", what,
                   bytes, w ? w->size : (size_t)0);
        return nullptr;
    }
    cudaGetLastError();
    if (w && w->ptr) {
        cudaStreamSynchronize(as_stream(stream));
        cudaFree(w->ptr);
        w->ptr = nullptr;
        w->size = 0;
    }
    size_t want = bytes < floor ? floor : bytes;
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_status(GB_ERR_OOM, "%s: cudaMalloc(%zu) failed: %s", what, want, cudaGetErrorString(e));
        return nullptr;
    }
    if (zero && (e = cudaMemsetAsync(p, 0, want, as_stream(stream))) != cudaSuccess) {
        cudaFree(p);
        set_status(GB_ERR_CUDA, "%s: cudaMemsetAsync failed: %s", what, cudaGetErrorString(e));
        return nullptr;
    }
    if (!w) {
        pool.push_back(WsEntry{dev, stream, nullptr, 0, 0});
        w = &pool.back();
    }
    w->ptr = p;
    w->size = want;
    if (size) *size = want;
    return p;
}

void *workspace(size_t bytes, void *stream) { return pool_buffer(g_ws, bytes, stream, size_t(64) << 20, "workspace"); }

// small per-stream scratch of the error report, apart from the GEMM workspace
static std::vector<WsEntry> g_aux;
void *aux_buffer(size_t bytes, void *stream) { return pool_buffer(g_aux, bytes, stream, size_t(64) << 10, "aux"); }

// per-stream line maxima of the FP16 form (cleared when made; only scans write it)
static std::vector<WsEntry> g_lm;
void *linemax_buffer(size_t bytes, void *stream, size_t *size) {
    return pool_buffer(g_lm, bytes, stream, size_t(64) << 10, "line maxima", true, size);
}

// The error word lives in a file-scope device variable (zero when the module
// loads), so finding it needs no allocation: its device address is looked up
// once per device, with that device current.
static __device__ int g_err_word_dev;
static int *g_err_word[kMaxDev] = {nullptr};

int *error_word() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDev) return nullptr;
    std::lock_guard<std::mutex> lk(g_ws_mu);
    if (!g_err_word[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_err_word_dev) != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return nullptr;
        }
        g_err_word[dev] = (int *)p;
    }
    return g_err_word[dev];
}

// ------------------------------------------------------------ self-test
// One thread waits on an mbarrier that nothing arrives at, through the same
// bounded wait the TMA / tensor-core kernels use, with a caller-given limit:
// the wait gives up, records code 99 in the error word and the kernel
// returns.  Nothing else is in flight (no TMA, no tensor memory).
__global__ void bounded_wait_selftest_kernel(int *err, uint64_t limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    ptx::mbar_init(&bar, 1);
    ptx::fence_mbar_init();
    ptx::mbar_wait_limit(&bar, 0, err, 99, limit_ns);
}

// ------------------------------------------------------------ FMA peak
// Eight independent FMA chains per thread, 16 steps each per iteration, on
// every SM: the scalar FP32 (FFMA) or FP64 (DFMA) throughput of this GPU,
// the roofline of the plain SIMT kernels.  x -> x*a + b with a = 1 - 2^-20,
// b = 2^-20 keeps every chain near 1; the sum is stored only if it takes an
// impossible value, so the chains are not removed.
static __device__ float g_fma_sink32;
static __device__ double g_fma_sink64;

template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = (T)1 + (T)(threadIdx.x + j) * (T)1e-7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int s = 0; s < 16; s++)
#pragma unroll
            for (int j = 0; j < 8; j++) x[j] = fma(x[j], a, b);
    }
    T sum = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) sum += x[j];
    if (sum == (T)-12345) {
        if (sizeof(T) == 8) g_fma_sink64 = (double)sum;
        else g_fma_sink32 = (float)sum;
    }
}

template <typename T>
static gb_status fma_peak(double *tflops, void *stream) {
    cudaStream_t st = as_stream(stream);
    const int blocks = sm_count() * 8, threads = 256;
    const int iters = sizeof(T) == 8 ? 256 : 4096;
    cudaEvent_t e0, e1;
    GB_CUDA_TRY(cudaEventCreate(&e0));
    GB_CUDA_TRY(cudaEventCreate(&e1));
    const T a = (T)1 - (T)(1.0 / 1048576.0), b = (T)(1.0 / 1048576.0);
    fma_peak_kernel<T><<<blocks, threads, 0, st>>>(iters / 8, a, b);   // warm-up
    GB_LAUNCH_CHECK("fma_peak_kernel");
    GB_CUDA_TRY(cudaEventRecord(e0, st));
    fma_peak_kernel<T><<<blocks, threads, 0, st>>>(iters, a, b);
    GB_LAUNCH_CHECK("fma_peak_kernel");
    GB_CUDA_TRY(cudaEventRecord(e1, st));
    GB_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    GB_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return ok();
}

// -------------------------------------------------------------- generator
template <typename T>
__global__ void fill_kernel(T *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind) {
    const uint64_t s = mix64(seed);
    const uint64_t s2 = mix64(seed ^ 0x5851F42D4C957F2DULL);
    const int64_t total = rows * cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t idx = (uint64_t)i;
        uint64_t b = mix64(s + (idx + 1) * 0x9E3779B97F4A7C15ULL);
        double u = (double)(b >> 11) * 0x1.0p-53;
        double v;
        if (kind == 1) {
            v = u;
        } else {
            v = 2.0 * u - 1.0;
            if (kind == 2) {
                uint64_t be = mix64(s2 + (idx + 1) * 0x9E3779B97F4A7C15ULL);
                int e = (int)(be % 41ULL) - 20;
                v = ldexp(v, e);
            }
        }
        int64_t r = i / cols, c = i - r * cols;
        X[r * ld + c] = (T)v;
    }
}

template <typename T>
static gb_status fill(T *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind, void *stream) {
    GB_CHECK_ARG(rows >= 0 && cols >= 0, "fill: negative size");
    GB_CHECK_ARG(ld >= cols, "fill: ld (%lld) < cols (%lld)", (long long)ld, (long long)cols);
    GB_CHECK_ARG(kind >= 0 && kind <= 2, "fill: kind %d not in 0..2", kind);
    if (rows == 0 || cols == 0) return ok();
    GB_CHECK_ARG(X != nullptr, "fill: null pointer");
    int64_t total = rows * cols;
    int blocks = (int)(total / 256 + 1 < (int64_t)sm_count() * 16 ? total / 256 + 1 : (int64_t)sm_count() * 16);
    fill_kernel<T><<<blocks, 256, 0, as_stream(stream)>>>(X, rows, cols, ld, seed, kind);
    GB_LAUNCH_CHECK("fill_kernel");
    return ok();
}

}  // namespace gb

using namespace gb;

extern "C" {

const char *gb_status_string(int status) {
    switch (status) {
        case GB_OK: return "GB_OK";
        case GB_ERR_INVALID_ARG: return "GB_ERR_INVALID_ARG";
        case GB_ERR_UNSUPPORTED: return "GB_ERR_UNSUPPORTED";
        case GB_ERR_OOM: return "GB_ERR_OOM";
        case GB_ERR_DEVICE_TIMEOUT: return "GB_ERR_DEVICE_TIMEOUT";
        case GB_ERR_CUDA: return "GB_ERR_CUDA";
        case GB_ERR_NO_DEVICE: return "GB_ERR_NO_DEVICE";
        default: return "GB_ERR_UNKNOWN";
    }
}

int gb_get_last_status(void) { return t_status; }
const char *gb_last_error(void) { return t_msg; }
const char *gb_last_error_string(void) { return t_msg; }
void gb_clear_last_status(void) {
    t_status = GB_OK;
    t_msg[0] = 0;
}

int gb_version(void) { return 100; }

uint64_t gb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int gb_device_arch(void) {
    int dev = 0, maj = 0, min = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&min, cudaDevAttrComputeCapabilityMinor, dev);
    return maj * 10 + min;
}

gb_status gb_sync(void *stream) {
    GB_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < kMaxDev && g_err_word[dev]) {
        int code = 0;
        GB_CUDA_TRY(cudaMemcpy(&code, g_err_word[dev], sizeof(int), cudaMemcpyDeviceToHost));
        if (code != 0) {
            cudaMemset(g_err_word[dev], 0, sizeof(int));
            return set_status(GB_ERR_DEVICE_TIMEOUT, "a device-side wait gave up (code %d)", code);
        }
    }
    return ok();
}

gb_status gb_malloc(void **ptr, size_t bytes) {
    GB_CHECK_ARG(ptr != nullptr, "gb_malloc: null out-pointer");
    *ptr = nullptr;
    if (bytes == 0) return ok();
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_status(GB_ERR_OOM, "gb_malloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return ok();
}

gb_status gb_malloc_managed(void **ptr, size_t bytes) {
    GB_CHECK_ARG(ptr != nullptr, "gb_malloc_managed: null out-pointer");
    *ptr = nullptr;
    if (bytes == 0) return ok();
    cudaError_t e = cudaMallocManaged(ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_status(GB_ERR_OOM, "gb_malloc_managed(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return ok();
}

gb_status gb_free(void *ptr) {
    if (ptr) GB_CUDA_TRY(cudaFree(ptr));
    return ok();
}

gb_status gb_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream) {
    GB_CHECK_ARG(kind >= 0 && kind <= 2, "gb_memcpy: kind %d not in 0..2", kind);
    if (bytes == 0) return ok();
    GB_CHECK_ARG(dst && src, "gb_memcpy: null pointer");
    cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost
                                                                      : cudaMemcpyDeviceToDevice;
    GB_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, k, as_stream(stream)));
    return ok();
}

gb_status gb_workspace_reserve(size_t bytes, void *stream) {
    if (bytes == 0) return ok();
    if (!workspace(bytes, stream)) return (gb_status)gb_get_last_status();
    // the FP16 form's line maxima: 2 x 8 bytes per line, at most bytes / 512 lines
    size_t got = 0;
    if (!linemax_buffer(bytes / 32, stream, &got)) return (gb_status)gb_get_last_status();
    return ok();
}

gb_status gb_selftest_bounded_wait(uint64_t limit_ns, void *stream) {
    GB_CHECK_ARG(limit_ns >= 1000 && limit_ns <= 100000000ull,
                 "gb_selftest_bounded_wait: limit %llu ns not in [1 us, 100 ms]", (unsigned long long)limit_ns);
    int *err = error_word();
    if (!err) return set_status(GB_ERR_CUDA, "gb_selftest_bounded_wait: no device error word");
    bounded_wait_selftest_kernel<<<1, 32, 0, as_stream(stream)>>>(err, limit_ns);
    GB_LAUNCH_CHECK("bounded_wait_selftest_kernel");
    return ok();
}

gb_status gb_measure_fma_peak(int dtype_bits, double *tflops, void *stream) {
    GB_CHECK_ARG(dtype_bits == 32 || dtype_bits == 64, "gb_measure_fma_peak: dtype_bits must be 32 or 64");
    GB_CHECK_ARG(tflops != nullptr, "gb_measure_fma_peak: null out-pointer");
    return dtype_bits == 64 ? fma_peak<double>(tflops, stream) : fma_peak<float>(tflops, stream);
}

gb_status gb_fill_f64(double *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind, void *stream) {
    return fill<double>(X, rows, cols, ld, seed, kind, stream);
}

gb_status gb_fill_f32(float *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind, void *stream) {
    return fill<float>(X, rows, cols, ld, seed, kind, stream);
}

}  // extern "C"
