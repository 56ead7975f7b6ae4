/*
 * gbblas.h -- C ABI of the GB300 (sm_103a) BLAS hot path.
 *
 * A drop-in for the GEMM / transpose / Jacobi path of
 * VVinstonSmith/BLAS-for-multi-core-DSP.  Conventions follow the reference:
 * row-major storage, OFFSET(row, col, ld) = row*ld + col; an operand used
 * transposed is stored transposed (op(A) = A^T means A is a K x M buffer,
 * lda >= M).  All pointers are device pointers (cudaMalloc, cudaMallocManaged
 * or any device-visible allocation) unless a function says otherwise.  The
 * library never frees caller memory.
 *
 * Calls are stream-ordered and asynchronous on the stream given (NULL: the
 * legacy default stream); gb_sync() waits for a stream.  Every entry point
 * returns a gb_status; the reference-named wrappers (gbblas_ref.h) return
 * void, as the reference does, and record their status for
 * gb_get_last_status().  Status and error text are per host thread.
 *
 * Plain pointers and integers only: no CUDA or torch types in signatures.
 */
#ifndef GBBLAS_H
#define GBBLAS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status */
typedef enum gb_status {
    GB_OK = 0,
    GB_ERR_INVALID_ARG = 1,    /* bad size, leading dimension, pointer, mode */
    GB_ERR_UNSUPPORTED = 2,    /* valid request this build cannot run        */
    GB_ERR_OOM = 3,            /* device allocation failed / over budget      */
    GB_ERR_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up          */
    GB_ERR_CUDA = 5,           /* CUDA runtime error (text in gb_last_error)  */
    GB_ERR_NO_DEVICE = 6       /* no usable sm_103 device                     */
} gb_status;

const char *gb_status_string(int status);
/* Status and message of the last failing call on this host thread. */
int         gb_get_last_status(void);
const char *gb_last_error(void);
const char *gb_last_error_string(void);   /* the same message (alias) */
void        gb_clear_last_status(void);

/* Library version and the device it runs on (major*10+minor, e.g. 103). */
int gb_version(void);
int gb_device_arch(void);

/* Kernel launches the library has issued so far (all threads). */
uint64_t gb_launch_count(void);

/* Stream-ordered completion; NULL = legacy default stream. */
gb_status gb_sync(void *stream);

/* Device memory helpers (cudaMalloc / cudaFree / cudaMemcpy wrappers) so a
 * C caller needs no CUDA headers.  kind: 0 host->device, 1 device->host,
 * 2 device->device (asynchronous on `stream`). */
gb_status gb_malloc(void **ptr, size_t bytes);
/* Memory visible to host and device (cudaMallocManaged); free with gb_free. */
gb_status gb_malloc_managed(void **ptr, size_t bytes);
gb_status gb_free(void *ptr);
gb_status gb_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream);

/* The library keeps one grow-only scratch buffer per (device, stream) for
 * split-K partials and split / sliced GEMM operands.  Growing it
 * synchronises that stream; reserve the largest size up front to keep
 * cudaMalloc off the call path of later calls on `stream`.  Calls captured
 * into a CUDA graph refer to the buffer as it was at capture: reserve it
 * before capturing, and do not let later calls on that stream grow it while
 * the graph is still replayed (growing frees the old buffer). */
gb_status gb_workspace_reserve(size_t bytes, void *stream);

/* Self-test of the bounded device waits (no reference counterpart; the
 * reference's kernels have no waits that can give up).  Every mbarrier wait
 * of the TMA / tensor-core kernels gives up after 2 s, records a code in a
 * per-device error word, and the kernel winds down; gb_sync() then returns
 * GB_ERR_DEVICE_TIMEOUT and clears the word.  This call runs one such wait on
 * a barrier that nothing arrives at, with a limit of limit_ns (1 us .. 100
 * ms), so that it gives up: the next gb_sync() on `stream` returns
 * GB_ERR_DEVICE_TIMEOUT, the one after that GB_OK, and the device stays
 * usable. */
gb_status gb_selftest_bounded_wait(uint64_t limit_ns, void *stream);

/* Scalar FMA throughput of the current device (no reference counterpart): a
 * short kernel of independent FFMA (dtype_bits 32) or DFMA (64) chains on
 * every SM, timed with CUDA events on `stream`; *tflops = 2 x FMAs / time.
 * The roofline of the plain SIMT / DFMA kernels.  Synchronises `stream`. */
gb_status gb_measure_fma_peak(int dtype_bits, double *tflops, void *stream);

/* ------------------------------------------------------------ inputs */
/* Seeded counter-based generator (bit-identical to the oracle's): element
 * (r,c) of a rows x cols matrix (leading dimension ld) gets f(seed, r*cols+c).
 * kind 0: U[-1,1], 1: U[0,1], 2: ldexp(U[-1,1], e) with e ~ U{-20..20}. */
gb_status gb_fill_f64(double *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind, void *stream);
gb_status gb_fill_f32(float *X, int64_t rows, int64_t cols, int64_t ld, uint64_t seed, int kind, void *stream);

/* ------------------------------------------------------------- GEMM */
typedef enum gb_algo {
    GB_ALGO_AUTO = 0,     /* pick per shape and dtype                          */
    GB_ALGO_ORDERED = 1,  /* the reference's summation order, bit-exact         */
    GB_ALGO_SIMT = 2,     /* plain FP32 FFMA / FP64 DFMA register tiles         */
    GB_ALGO_DMMA = 3,     /* FP64 tensor pipe (mma.sync m8n8k4 f64)             */
    GB_ALGO_BF16X3 = 4,   /* SGEMM as hi*hi+hi*lo+lo*hi BF16 on tcgen05, FP32 acc */
    GB_ALGO_OZAKI = 5,    /* DGEMM from exact integer slices on tensor cores    */
    GB_ALGO_SKINNY = 6,   /* tiny M (shortA) / tiny N (thinB) streaming kernels */
    GB_ALGO_BF16X6 = 7,   /* SGEMM from 3 BF16 pieces (6 products) on tcgen05:
                             FP32-level error at half the BF16X3 rate        */
    GB_ALGO_FP16X3 = 8    /* SGEMM from 2 FP16 pieces of power-of-two scaled
                             rows of op(A) / columns of op(B) (3 products,
                             folded accumulation) on tcgen05: FP32-level
                             error                                            */
} gb_algo;

typedef enum gb_semantics {
    /* C = alpha*op(A)op(B) + beta*C (BLAS; beta == 0: C is not read).  With
     * alpha == beta == 1 and GB_ALGO_ORDERED this is the reference DGEMM /
     * irregular V0.0 update C += op(A)op(B) in its order. */
    GB_SEM_BLAS = 0,
    /* C = alpha*op(A)op(B) + beta, beta a scalar added to every element, C not
     * read (sgemm_release_V1.3.2, irr_thinB_sgemm_release_V1.2). */
    GB_SEM_SCALAR_BETA = 1,
    /* C = C + alpha*op(A)op(B) + beta (sgemm_release_V1.3.1). */
    GB_SEM_ACCUM_SCALAR_BETA = 2
} gb_semantics;

typedef struct gb_gemm_opts {
    void   *stream;        /* cudaStream_t; NULL = legacy default stream       */
    int32_t algo;          /* gb_algo                                          */
    int32_t semantics;     /* gb_semantics                                     */
    int32_t k_block;       /* ORDERED: outer K block (reference K_G), 0 -> 512  */
    int32_t k_slab;        /* ORDERED: inner K slab (K_A, three-level sum of
                              irr_thinB_sgemm V1.2), 0 -> two-level sum        */
    int32_t alpha_on_b;    /* ORDERED: alpha pre-scales op(B) (thinB V1.2)
                              instead of op(A) (sgemm V1.3.x)                  */
    int32_t ozaki_slices;  /* OZAKI: 8-bit (balanced) slices per operand
                              (2..9), 0 -> the fewest meeting target_err      */
    double  target_err;    /* OZAKI: normwise error target, 0 -> no worse
                              than native FP64 (8 slices)                     */
    int32_t accum_k;       /* BF16X3 / BF16X6 / FP16X3: restart the tensor-
                              memory accumulator every accum_k values of K
                              (rounded up to 32) and sum the parts in FP32
                              registers; 0 -> the form's default (FP16X3 128,
                              BF16X6 256, BF16X3 never); < 0 -> never         */
    int32_t split_k;       /* SKINNY: number of K ranges computed apart and
                              summed (split-K); 0 -> the planner's choice     */
    double *err_out;       /* non-NULL: after the product, in stream order,
                              store its normwise error estimate here (memory
                              the device writes: device, managed or mapped
                              pinned host memory):
                              ||C - C*||_F / (|alpha| ||op(A)_I||_F
                              ||op(B)_J||_F + |beta| ||C0_IJ||_F) over 16
                              rows I and 16 columns J spread evenly over C
                              (all when M or N < 16), C* by Dot2 rounded to
                              FP64; scalar-beta semantics use |beta|
                              sqrt(|I||J|) (+ ||C0_IJ||_F when accumulating)
                              for the last term.  Two extra launches; the
                              buffer they share is per stream (64 KB, made
                              on first use: before a graph capture, make one
                              call with err_out on the stream)              */
} gb_gemm_opts;

/* Fill *opts with defaults (AUTO, BLAS, NULL stream). */
void gb_gemm_opts_init(gb_gemm_opts *opts);

/* transA/transB: 'N' or 'T' (case-insensitive).  Shapes: op(A) is M x K,
 * op(B) is K x N, C is M x N.  lda >= (transA=='N' ? K : M),
 * ldb >= (transB=='N' ? N : K), ldc >= N.  M, N or K == 0 is valid
 * (K == 0 still applies beta).  opts may be NULL.
 * Stream-ordered: work queued after a call sees its C.  Two BF16X3 / BF16X6
 * calls back to back on one stream may overlap the second's operand split
 * with the first's GEMM (never its GEMM with the first's) when the second's
 * A and B do not overlap the first's C; work queued on the stream between
 * the two calls is waited for before the split reads A and B.  FP64 through the
 * digit forms (OZAKI, FP64 SKINNY): an output whose row of op(A) or column of
 * op(B) holds an Inf or a NaN is computed as a plain FP64 dot product, so
 * they propagate as in IEEE arithmetic. */
gb_status gb_sgemm(char transA, char transB, int64_t M, int64_t N, int64_t K,
                   float alpha, const float *A, int64_t lda, const float *B, int64_t ldb,
                   float beta, float *C, int64_t ldc, const gb_gemm_opts *opts);
gb_status gb_dgemm(char transA, char transB, int64_t M, int64_t N, int64_t K,
                   double alpha, const double *A, int64_t lda, const double *B, int64_t ldb,
                   double beta, double *C, int64_t ldc, const gb_gemm_opts *opts);

/* Skinny FP32 GEMM that allocates no device memory.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc on the call
 * path -- a serving loop that admits work against a fixed HBM budget, a host
 * framework whose device memory belongs to its own pool allocator, or code
 * that must not trigger the device-wide synchronisation cudaFree implies.
 * For min(M, N) <= 8 it computes exactly what gb_sgemm with GB_ALGO_SKINNY
 * computes (same kernels, same split-K plan; thinB when N <= M, else
 * shortA); for 8 < min(M, N) <= 64, where GB_ALGO_SKINNY runs 3xBF16 on the
 * tensor cores, it runs the FP32 FFMA streaming kernels (FP32 rounding, the
 * same 2*K*u normwise bound).  K >= 1.  It keeps the split-K partial sums
 * (and, when an operand's layout cannot be read by TMA in place, a packed copy
 * of the small operand) in a fixed
 * 16 MiB array of device memory that every GPU loading the library reserves
 * until the process exits.  A call whose split-K plan needs more than 16 MiB
 * (splits x max(M, N) x padded min(M, N) x 4 bytes) is rejected with
 * GB_ERR_INVALID_ARG before anything runs.  The first call on each device
 * looks up the device addresses of that array and of the library's device
 * error word (both file-scope device variables, found with
 * cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share
 * the one array: calls that overlap on the GPU (different streams, or
 * different host threads) race on it and must be serialised by the caller.
 * `semantics` is a gb_semantics value; `stream` as in gb_gemm_opts. */
gb_status gb_sgemm_skinny_noalloc(char transA, char transB, int64_t M, int64_t N, int64_t K,
                                  float alpha, const float *A, int64_t lda, const float *B, int64_t ldb,
                                  float beta, float *C, int64_t ldc, int semantics, void *stream);

/* Algorithm that GB_ALGO_AUTO picks for a shape (for logging/tests). */
int gb_gemm_pick_algo(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K);

/* Workspace bytes (the library-owned scratch of the call's stream) that the
 * gb_sgemm (dtype_bits 32) / gb_dgemm (64) call with these arguments and
 * options may use (no reference counterpart: the reference's kernels work in
 * fixed on-chip buffers, e.g. the static GSM array of
 * sgemm_release_V1.3.2/device_code/sgemm_kernel.c:17): the 16-bit operand pieces of BF16X3 / BF16X6 / FP16X3, the
 * skinny products' split-K parts, the Ozaki slices; 0 for the forms that need
 * none.  opts as the call's (NULL: the defaults; algo AUTO resolves as the
 * call would; ozaki_slices 0 takes the count target_err picks); A and B are
 * read only for their alignment, and NULL stands for 16-byte aligned.  The
 * Ozaki figure includes scratch per SM of the current device: query with the
 * device that will run the call current.
 * Reserving the figure with gb_workspace_reserve before capturing such a call
 * into a CUDA graph keeps the capture from needing to grow the buffer. */
gb_status gb_workspace_query(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                             const void *A, int64_t lda, const void *B, int64_t ldb,
                             const gb_gemm_opts *opts, size_t *bytes);

/* ------------------------------------------------------ grouped GEMM */
/* One GEMM of a batch (same meaning as the gb_sgemm / gb_dgemm arguments). */
typedef struct gb_gemm_desc {
    int32_t dtype_bits;      /* 32 (FP32) or 64 (FP64)                       */
    char    transA, transB;  /* 'N' or 'T'                                   */
    char    pad[2];
    int32_t semantics;       /* gb_semantics                                 */
    int32_t reserved;
    int64_t M, N, K;
    double  alpha, beta;
    const void *A; int64_t lda;
    const void *B; int64_t ldb;
    void       *C; int64_t ldc;
} gb_gemm_desc;

/* Run n independent GEMMs of any shapes, modes, semantics and dtypes
 * (FP32 / FP64 mixed) in one launch of a persistent grouped kernel: the
 * descriptors become a device work list and every CTA pulls 64 x 64 C tiles
 * from the whole batch, so many small problems fill the GPU together.  No
 * reference counterpart (the reference runs one problem per DSP cluster);
 * it is the batching layer of the serving path.  n <= 4096.  Asynchronous
 * on `stream`; the descriptors are copied before the call returns. */
gb_status gb_gemm_batch(const gb_gemm_desc *descs, int n, void *stream);

/* Strided batch of equal-shape GEMMs: GEMM i reads A + i*strideA and
 * B + i*strideB and writes C + i*strideC (strides in elements; 0 shares an
 * operand), each as in gb_sgemm / gb_dgemm (dtype_bits 32 or 64), through
 * the grouped kernel in launches of up to 4096.  No reference counterpart
 * (ld-aware batched variants of the irregular path). */
gb_status gb_gemm_strided_batched(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                                  double alpha, const void *A, int64_t lda, int64_t strideA,
                                  const void *B, int64_t ldb, int64_t strideB, double beta,
                                  void *C, int64_t ldc, int64_t strideC, int64_t batch, int semantics,
                                  void *stream);

/* ------------------------------------------------------ transpose */
/* B (N x M, ldb >= M) = A^T, A is M x N (lda >= N).  Bit-exact copy.
 * Replaces transpose/device_code/kernel.c:2002 transpose_float_32x32_dbuf
 * and :1167 transpose_16x16_dbuf, and dgemm_kernel.c:974 transpose_A2B. */
gb_status gb_transpose_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb, void *stream);
gb_status gb_transpose_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb, void *stream);

/* B (N x M, ldb >= M) += A^T, A is M x N (lda >= N): one IEEE add per
 * element, bit-exact.  The transpose-accumulate of the reference's
 * micro_kernel_16x16_add / micro_kernel_16x16x2_add (dgemm_release_V1.1/
 * device_code/dgemm_kernel.c:174, :635) and micro_kernel_float_32x32_add
 * (sgemm_release_V1.3.1/device_code/sgemm_kernel.c:482) as an entry point. */
gb_status gb_transpose_add_f32(int64_t M, int64_t N, const float *A, int64_t lda, float *B, int64_t ldb,
                               void *stream);
gb_status gb_transpose_add_f64(int64_t M, int64_t N, const double *A, int64_t lda, double *B, int64_t ldb,
                               void *stream);

/* -------------------------------------------------------- stencil */
typedef enum gb_stencil_order {
    GB_STENCIL_HOST = 0,   /* ((((top+left)+right)+down)+middle)*0.2 (matrix_stencil.c:45)  */
    GB_STENCIL_SCALAR = 1, /* 0.2*((((top+middle)+down)+left)+right) (kernel_stencil.c:70)  */
    GB_STENCIL_VECTOR = 2  /* row-parity add tree of micro_kernel_cross_reduce_V3          */
} gb_stencil_order;

/* `iters` 5-point Jacobi sweeps on (M+2) x (N+2) padded grids A and B
 * (row stride N+2), ping-ponging: sweep 1 reads A writes B, sweep 2 reads B
 * writes A, ...  Halo cells are never written (Dirichlet boundary: set it in
 * both buffers).  The result is in B when iters is odd, in A when even;
 * the interior of the other buffer is scratch (sweeps are fused several per
 * launch, so it holds some earlier sweep, not necessarily iters-1).
 * iters == 1 is the reference stencil_vector(M, N, A, B)
 * (stencil_2d_V1.2/device_code/kernel_stencil.c:1042).  Bit-exact for the
 * chosen order. */
gb_status gb_stencil2d_f64(int64_t M, int64_t N, double *A, double *B, int iters, int order, void *stream);
gb_status gb_stencil2d_f32(int64_t M, int64_t N, float *A, float *B, int iters, int order, void *stream);

/* `iters` sweeps of a 9-point stencil with the 3x3 weight window w (a HOST
 * array of 9: w[0..2] weigh the row above (columns -1, 0, +1), w[3..5] the
 * row itself, w[6..8] the row below), on the same padded grids, ping-pong
 * and fixed halo as gb_stencil2d:
 *     r = w0*a(-1,-1); r = fma(w1, a(-1,0), r); ... r = fma(w8, a(+1,+1), r)
 * in window order, so results are bit-identical to that recurrence.  No
 * reference counterpart: the generalisation of stencil_2d
 * (stencil_2d_V1.2/device_code/kernel_stencil.c) on the same temporal-
 * blocking engine. */
gb_status gb_stencil9_f32(int64_t M, int64_t N, float *A, float *B, int iters, const float *w, void *stream);
gb_status gb_stencil9_f64(int64_t M, int64_t N, double *A, double *B, int iters, const double *w, void *stream);

/* ---------------------------------------------------------- serving */
/* A request loop over the kernels above, for streams of independent
 * problems: operands stay device-resident (the caller owns them), requests
 * are admitted while the bytes of all in-flight requests fit an HBM budget
 * (FIFO; a request larger than the whole budget is rejected with
 * GB_ERR_OOM), small GEMMs admitted together run in one grouped launch
 * (replayed from CUDA graphs), the rest run one launch each with the
 * algorithm the autotune table picks (captured into a CUDA graph per
 * bucket and replayed), over a pool of streams.  Latency is
 * measured from submit to the completion callback on the stream.  No
 * reference counterpart (the reference host runs one kernel at a time). */
typedef enum gb_op { GB_OP_GEMM = 0, GB_OP_TRANSPOSE = 1, GB_OP_STENCIL = 2 } gb_op;

typedef struct gb_request {
    int32_t op;              /* gb_op                                                 */
    int32_t dtype_bits;      /* 32 or 64                                              */
    char    transA, transB;  /* GEMM modes                                            */
    char    pad[2];
    int32_t algo;            /* GEMM gb_algo; AUTO = autotune table, then heuristic    */
    int32_t semantics;       /* GEMM gb_semantics                                     */
    int32_t iters, order;    /* stencil sweeps and gb_stencil_order                   */
    int32_t reserved;
    int64_t M, N, K;         /* GEMM op(A) M x K, op(B) K x N; transpose A M x N;
                                stencil interior M x N                                */
    double  alpha, beta;     /* GEMM                                                  */
    const void *A; int64_t lda;   /* GEMM A / transpose source / stencil grid A      */
    void       *B; int64_t ldb;   /* GEMM B / transpose destination                  */
    void       *C; int64_t ldc;   /* GEMM C / stencil grid B                         */
    uint64_t bytes;          /* HBM charge while in flight (0: its operand bytes)     */
    uint64_t tag;            /* returned by gb_server_poll                            */
} gb_request;

typedef struct gb_server_config {
    uint64_t hbm_budget_bytes;  /* admission budget (default 48 GiB)                  */
    uint64_t workspace_bytes;   /* scratch reserved per stream at creation (0: grow)  */
    double   group_max_work;    /* GEMMs with M*N*K <= this, min(M,N) > 64 and algo
                                   AUTO go to grouped launches (default 512^3)        */
    int32_t  streams;           /* device streams (default 6)                         */
    int32_t  max_batch;         /* GEMMs per grouped launch (default 256)             */
    int32_t  max_inflight;      /* requests in flight at once (default 2^20)          */
    int32_t  use_graphs;        /* replay launches from CUDA graphs (1): grouped
                                   launches per slot, one-launch requests per
                                   (op, dtype, modes, algorithm, log2 sizes) bucket,
                                   the stream's workspace grown to the request's
                                   bound before each capture                         */
    int32_t  use_grouped;       /* group small GEMMs (1); 0 = one launch per request  */
    int32_t  dry_run;           /* admission and bookkeeping only, no device work     */
    double   short_us;          /* requests estimated below this many microseconds
                                   (and grouped launches) go round-robin to the
                                   first short_streams streams, created at the
                                   device's highest priority, the rest round-robin
                                   over the others, so that short work is not
                                   queued behind long kernels (default 200; 0: one
                                   pool, no priorities)                             */
    int32_t  short_streams;     /* high-priority streams (default 2; at most
                                   streams - 1 are used)                            */
    int32_t  long_sm_percent;   /* long requests plan their persistent grids for
                                   this share of the SMs, leaving the rest to short
                                   work (1..100; default 100: all)                  */
} gb_server_config;

typedef struct gb_server_stats {
    int64_t  submitted, completed, rejected, failed, waiting, inflight;
    uint64_t inflight_bytes;
    int64_t  launches, grouped_launches, grouped_requests;
    double   p50_s, p99_s, mean_s, req_per_s;
    int64_t  graph_launches;        /* launches that replayed a CUDA graph (grouped and one-launch)    */
    int64_t  graph_instantiations;  /* one-launch graphs built (the rest were cached graphs updated)   */
    int64_t  urgent_launches;       /* launches on the high-priority streams (short requests, groups) */
} gb_server_stats;

typedef struct gb_server gb_server;

void      gb_server_config_init(gb_server_config *cfg);
gb_status gb_server_create(const gb_server_config *cfg, gb_server **out);
/* Queue a request (returns at once; the operands must stay valid until the
 * request's tag is returned by gb_server_poll or gb_server_drain returns). */
gb_status gb_server_submit(gb_server *s, const gb_request *req);
/* Completed requests since the last poll: tags and latencies (seconds). */
int       gb_server_poll(gb_server *s, uint64_t *tags, double *latency_s, int max);
/* Wait until every submitted request completed (timeout_s <= 0: no limit). */
gb_status gb_server_drain(gb_server *s, double timeout_s);
gb_status gb_server_get_stats(gb_server *s, gb_server_stats *out);
void      gb_server_destroy(gb_server *s);

/* Autotuner.  No reference counterpart; the reference's tuning surface is
 * its per-mode blocking constants (sgemm_release_V1.3.2/device_code/
 * sgemm_kernel.c:2480-2493, the K_A / K_G table of
 * dgemm_release_V1.1/readme.txt:17-24, the r6c96 / r6c128 switch at
 * sgemm_kernel.c:14-15).  A choice is an algorithm and its knobs; the table
 * keeps one per (dtype, modes, log2 M, log2 N, log2 K) bucket, and
 * GB_ALGO_AUTO requests through the server use it. */
typedef struct gb_tune_choice {
    int32_t algo;          /* gb_algo                                         */
    int32_t accum_k;       /* as gb_gemm_opts.accum_k                         */
    int32_t split_k;       /* as gb_gemm_opts.split_k                         */
    int32_t ozaki_slices;  /* as gb_gemm_opts.ozaki_slices                    */
    double  ms;            /* median time of one call when it was measured    */
} gb_tune_choice;

/* Time every candidate for the shape on scratch operands (U[-1,1]) on
 * `stream` -- one warm-up call, then `reps` (>= 5; 0 -> 5) timed calls,
 * median taken, measured again when the spread of a candidate exceeds 30 % --
 * and record the fastest.  Candidates: FP32: SIMT, BF16X3 (K >= 64), FP16X3
 * with accumulator chunks of 128 and 256, BF16X6, and SKINNY (min(M, N) <=
 * 64) with the planner's split-K and 1, 4 and 16 splits; FP64: ORDERED,
 * DMMA, OZAKI with the fewest slices for `target_err` (0: no worse than
 * native FP64) and one more, SKINNY (min(M, N) <= 64).  Every FP32 candidate
 * meets the 2*K*u32 normwise bound; OZAKI meets target_err.  Synchronises
 * `stream`. */
gb_status gb_autotune_gemm_ex(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                              double target_err, int reps, void *stream, gb_tune_choice *best);
/* The same with reps 5, target_err 0, the legacy default stream. */
gb_status gb_autotune_gemm(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                           int *best_algo, double *best_ms);
/* Set a bucket's algorithm (knobs at their defaults) / read the full choice
 * of a bucket (returns GB_ERR_INVALID_ARG when the bucket has none). */
gb_status gb_autotune_set(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K, int algo);
gb_status gb_autotune_lookup(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                             gb_tune_choice *out);
/* The bucket's algorithm, -1 when the table has none. */
int       gb_autotune_get(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K);
/* Text file, one bucket per line: bits ta tb log2M log2N log2K algo accum_k split_k slices ms
 * (files with only the first seven columns load too). */
gb_status gb_autotune_save(const char *path);
gb_status gb_autotune_load(const char *path);

/* --------------------------------------------------- launch by name */
/* The reference host drives the device by kernel name with packed
 * arguments: hthread_group_exec(tg, "launch_sgemm_NN", n_scalar, n_ptr, args)
 * (sgemm_release_V1.3.2/host_code/sgemm_demo.c:144), scalars first then
 * pointers.  gb_exec runs the named reference kernel with the same packing
 * (names and argument lists of the reference launchers and device entries:
 * launch_dgemm_XX, launch_sgemm_XX, launch_irr_{shortA,thinB}_{s,d}gemm_XX,
 * transpose_float_32x32_dbuf, transpose_16x16_dbuf, stencil_vector, *_null)
 * and waits for it, as hthread_group_exec + hthread_group_wait do. */
gb_status gb_exec(const char *name, int n_scalar, int n_ptr, const unsigned long *args);

#ifdef __cplusplus
}
#endif
#endif
