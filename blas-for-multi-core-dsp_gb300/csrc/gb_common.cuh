// gb_common.cuh -- shared helpers of the GB300 BLAS library (host + device).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "gbblas.h"

namespace gb {

// ------------------------------------------------------------- status
// Records the status of the calling host thread (thread-local) and returns it.
gb_status set_status(gb_status st, const char *fmt, ...);
gb_status ok();
gb_status cuda_status(cudaError_t e, const char *where);

#define GB_CHECK_ARG(cond, ...)                                                \
    do {                                                                       \
        if (!(cond)) return ::gb::set_status(GB_ERR_INVALID_ARG, __VA_ARGS__); \
    } while (0)

#define GB_CUDA_TRY(expr)                                                      \
    do {                                                                       \
        cudaError_t _e = (expr);                                               \
        if (_e != cudaSuccess) return ::gb::cuda_status(_e, #expr);            \
    } while (0)

// Launch-error check after a kernel launch (asynchronous errors surface on
// the next synchronising call, as usual for CUDA).
#define GB_LAUNCH_CHECK(what)                                                  \
    do {                                                                       \
        ::gb::count_launch();                                                  \
        cudaError_t _e = cudaGetLastError();                                   \
        if (_e != cudaSuccess) return ::gb::cuda_status(_e, what);             \
    } while (0)

// Kernel launches issued by the library (all host threads).
void count_launch();

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int sm_count();
void set_sm_cap(int cap);   // this host thread's launches plan for at most cap SMs (0: all)
// Opt-in shared memory per block (bytes) of the current device.
int smem_optin();

// Scratch owned by the library, one grow-only buffer per (device, stream),
// guarded by a mutex.  Returns nullptr and sets GB_ERR_OOM on failure.  The
// buffer stays valid until the next call on the same stream needs more;
// work on that stream uses it in stream order.
void *workspace(size_t bytes, void *stream);
// The same, and *seq = the number of earlier calls of this form on the
// stream, *size = the buffer's size (>= bytes): callers that alternate
// between two halves of the buffer place them by *size, so that calls of
// different sizes never overlap each other's half.
void *workspace(size_t bytes, void *stream, unsigned *seq, size_t *size);
// small per-stream scratch (>= 64 KB), separate from the workspace
void *aux_buffer(size_t bytes, void *stream);
// per-stream buffer of the FP16 form's line maxima (cleared when made, *size = its bytes)
void *linemax_buffer(size_t bytes, void *stream, size_t *size);

// Per-device one-time setup (kernel attributes such as the dynamic shared
// memory limit hold per device): `done` has one bit per device.  Running the
// setup twice is harmless, so concurrent first calls may both do it.
bool device_setup_needed(const std::atomic<uint64_t> &done);
void device_setup_done(std::atomic<uint64_t> &done);

// Per-device error word (4 bytes of device memory, zero = no error) that
// kernels with bounded waits set on timeout; gb_sync() reports and clears it.
int *error_word();

inline bool is_trans(char t) { return t == 'T' || t == 't'; }
inline bool is_mode(char t) { return t == 'N' || t == 'n' || t == 'T' || t == 't'; }

#ifdef __CUDACC__
// Exponent of a line (row of X, column of W) that holds an Inf or a NaN:
// the digit paths (Ozaki DGEMM, FP64 skinny) take the line maximum's
// exponent, E - 1022 for biased exponent E, and E = 2047 only for Inf / NaN.
constexpr int kNonFiniteLineExp = 1025;

// e = smallest integer with max |x| < 2^e (0 for an all-zero line), from
// the maximum of the |x| bit patterns (monotone for non-negative doubles).
__device__ __forceinline__ int exp_of_maxbits(unsigned long long mb) {
    if (mb == 0) return 0;
    int E = (int)((mb >> 52) & 0x7FF);
    if (E == 0) {   // subnormal: value = m * 2^-1074, m < 2^52
        int lz = __clzll((long long)mb);      // m has 64 - lz significant bits
        return (64 - lz) - 1074;
    }
    return E - 1022;   // value in [2^(E-1023), 2^(E-1022))
}

// 2^k as a double for k >= -1022, 0 below
__device__ __forceinline__ double pow2_or_zero(int k) {
    return k >= -1022 ? __longlong_as_double((long long)(1023 + k) << 52) : 0.0;
}

// x * 2^k for |k| up to 3069 without a library call: up to three factors in
// the normal range, the largest first, so that only a result outside the
// normal range rounds.
__device__ __forceinline__ double mul_pow2(double x, int k) {
    const int a = max(-1022, min(1023, k));
    k -= a;
    const int b = max(-1022, min(1023, k));
    const int c = max(-1022, min(1023, k - b));
    return x * pow2_or_zero(a) * pow2_or_zero(b) * pow2_or_zero(c);
}

// Plain FP64 dot product of row `row` of X (rows x K; tx: stored K x rows)
// and column `col` of W (K x cols; tw: stored cols x K), in k order.  The
// digit paths use it for the outputs whose row or column holds an Inf or a
// NaN, so that those propagate as IEEE arithmetic has them.
__device__ inline double native_dot(const double *X, int64_t ldx, int tx, int64_t row, const double *W, int64_t ldw,
                                    int tw, int64_t col, int64_t K) {
    double s = 0.0;
    for (int64_t k = 0; k < K; k++) {
        const double x = tx ? X[k * ldx + row] : X[row * ldx + k];
        const double w = tw ? W[col * ldw + k] : W[k * ldw + col];
        s = fma(x, w, s);
    }
    return s;
}

// native_dot kept out of line, for the rare outputs that need it inside
// unrolled epilogue loops.
__device__ __noinline__ inline double native_dot_cold(const double *X, int64_t ldx, int tx, int64_t row,
                                                      const double *W, int64_t ldw, int tw, int64_t col, int64_t K) {
    return native_dot(X, ldx, tx, row, W, ldw, tw, col, K);
}
#endif

// Counter-based generator (identical to the oracle's gbo_* functions).
__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace gb

// ------------------------------------------------------------- launchers
// Internal kernel entry points (one per .cu file), called by the dispatchers.
namespace gb {

struct GemmArgs {
    bool ta, tb;
    int64_t M, N, K;
    const void *A; int64_t lda;
    const void *B; int64_t ldb;
    void *C; int64_t ldc;
    double alpha, beta;
    int semantics;   // gb_semantics
    int k_block, k_slab, alpha_on_b;
    int accum_k;     // tensor-core SGEMM forms: accumulator chunk in K (0 default, < 0 none)
    int split_k;     // skinny: split-K override (0: the planner's)
    cudaStream_t stream;
};

gb_status launch_gemm_ordered_f64(const GemmArgs &g);
gb_status launch_gemm_ordered_f32(const GemmArgs &g);
gb_status launch_sgemm_simt(const GemmArgs &g);
gb_status launch_dgemm_dmma(const GemmArgs &g);
gb_status launch_sgemm_bf16x3(const GemmArgs &g);
gb_status launch_sgemm_bf16x6(const GemmArgs &g);
gb_status launch_sgemm_fp16x3(const GemmArgs &g);
gb_status launch_dgemm_ozaki(const GemmArgs &g, int slices);
// Slice count (2..8) whose truncation error meets a normwise target for this K.
int ozaki_pick_slices(double target_err, int64_t K);
// Skinny FP32 product on the tensor cores (skinny_tc.cu): X rows x K (tx:
// stored K x rows), W K x n (tw: stored n x K), 8 < n <= nb in {16, 32, 64}.
struct ThinTcArgs {
    int64_t rows, K;
    const float *X; int64_t ldx; int tx;
    const float *W; int64_t ldw; int tw;
    int n, nb;
    float *C; int64_t cs_r, cs_c;
    float alpha, beta;
    int semantics;
    int splits; int64_t kchunk;                    // K range of a split: a multiple of 64
    float *part;                                   // splits x rows x nb partials (splits > 1)
    void *wpieces;                                 // thin_tc_wpieces_bytes(nb, K) of scratch
    cudaStream_t stream;
};
bool thin_tc_row_classes(int tx, int64_t ldx);          // row-major X with ldx % 4 != 0
int64_t thin_tc_stages(int64_t K, bool classes);       // 64-k stages per row tile
size_t thin_tc_wpieces_bytes(int nb, int64_t K, bool classes);
gb_status launch_thin_tc(const ThinTcArgs &a);

// FP64 skinny product from integer digits on the tensor cores (skinny_oz.cu).
bool thin_oz_eligible(int tx, int64_t ldx, const void *X, int64_t rows, int64_t K);
size_t thin_oz_workspace_bytes(int64_t rows, int64_t K, int n, int splits);
gb_status launch_thin_oz(int64_t rows, int64_t K, const double *X, int64_t ldx, int tx, const double *W, int64_t ldw,
                         int tw, int n, double *C, int64_t cs_r, int64_t cs_c, double alpha, double beta,
                         int semantics, int splits, int64_t kchunk, void *ws, cudaStream_t st);

gb_status launch_skinny_f32(const GemmArgs &g);
gb_status launch_skinny_f64(const GemmArgs &g);
size_t skinny_workspace_bytes(const GemmArgs &g, int bits);
// gemm_report.cu: the normwise error report around one product (before: norms and sampled C0;
// after: Dot2 of the sample against C, reduced into *out)
gb_status report_before(const GemmArgs &g, int bits);
gb_status report_after(const GemmArgs &g, int bits, double *out);   // what launch_skinny_* takes; launches nothing
// C = beta*C (beta==0: C = 0) or C = C + beta (scalar) epilogue-only path (K == 0)
gb_status launch_gemm_k0_f32(const GemmArgs &g);
gb_status launch_gemm_k0_f64(const GemmArgs &g);

}  // namespace gb
