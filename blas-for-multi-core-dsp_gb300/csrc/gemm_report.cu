// gemm_report.cu -- the per-call normwise error report of gb_sgemm /
// gb_dgemm (gb_gemm_opts.err_out).
//
// The reference's host demos check every result against a CPU loop
// (sgemm_release_V1.3.2/host_code/sgemm_demo.c:214-242, dgemm_demo.c:233-252);
// here a call may ask for the check on the device, on a fixed sample:
//
//   err = ||C_IJ - C*_IJ||_F / (|alpha| ||op(A)_I||_F ||op(B)_J||_F + t_IJ)
//
// over I = min(M, 16) rows and J = min(N, 16) columns spread evenly over C
// (row i of the sample is floor((2i+1) M / (2|I|))), C* the product
// evaluated with Dot2 (error-free transformations: TwoProduct by fma,
// TwoSum; Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26(6), 2005) and
// rounded once to FP64, and t_IJ the size of the added term:
// |beta| ||C0_IJ||_F (BLAS), |beta| sqrt(|I||J|) (scalar beta),
// ||C0_IJ||_F + |beta| sqrt(|I||J|) (accumulate).  For BLAS semantics this
// is the measure the test suite's oracle computes on the same rows and
// columns.
//
// Two launches around the product, in stream order: before it, the row and
// column norms and the sampled entries of C0 go to a small per-stream
// buffer; after it, one warp per sampled entry forms C* (each lane a strided
// part of K as a double-double, joined by TwoSum across the warp) and the
// last block to finish reduces the sample into *err_out.
#include "gb_common.cuh"

namespace gb {
namespace {

constexpr int kS = 16;   // sampled rows and columns (at most)

struct ReportBuf {
    double rn2[kS], cn2[kS];      // squared norms of the sampled rows of op(A) / columns of op(B)
    double c0[kS * kS];           // sampled C0
    double d2[kS * kS];           // squared difference of each sampled entry
    unsigned int done;            // blocks of the second launch that finished
};

struct ReportArgs {
    const void *A, *B, *C;
    int64_t lda, ldb, ldc, M, N, K;
    int ta, tb, nr, nc, semantics;
    double alpha, beta;
    ReportBuf *buf;
    double *out;
};

__device__ __forceinline__ int64_t sample_index(int i, int n, int64_t dim) {
    return ((2 * (int64_t)i + 1) * dim) / (2 * (int64_t)n);
}

template <typename T>
__device__ __forceinline__ double op_a(const ReportArgs &a, int64_t r, int64_t k) {
    const T *A = (const T *)a.A;
    return (double)(a.ta ? A[k * a.lda + r] : A[r * a.lda + k]);
}

template <typename T>
__device__ __forceinline__ double op_b(const ReportArgs &a, int64_t k, int64_t c) {
    const T *B = (const T *)a.B;
    return (double)(a.tb ? B[c * a.ldb + k] : B[k * a.ldb + c]);
}

// error-free transformations, with rounded-to-nearest operations the compiler may not contract
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
    s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(double a, double b, double &p, double &e) {
    p = __dmul_rn(a, b);
    e = fma(a, b, -p);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Blocks 0..nr-1: row norms; nr..nr+nc-1: column norms; the last: sampled C0
// and the completion counter.  32 threads each.
template <typename T>
__global__ void report_pre_kernel(ReportArgs a) {
    const int b = blockIdx.x, lane = threadIdx.x;
    ReportBuf *buf = a.buf;
    if (b < a.nr + a.nc) {
        const bool row = b < a.nr;
        const int64_t idx = row ? sample_index(b, a.nr, a.M) : sample_index(b - a.nr, a.nc, a.N);
        double s = 0.0;
        for (int64_t k = lane; k < a.K; k += 32) {
            const double v = row ? op_a<T>(a, idx, k) : op_b<T>(a, k, idx);
            s = __dadd_rn(s, __dmul_rn(v, v));
        }
        s = warp_sum(s);
        if (lane == 0) (row ? buf->rn2[b] : buf->cn2[b - a.nr]) = s;
        return;
    }
    const T *C = (const T *)a.C;
    for (int e = lane; e < a.nr * a.nc; e += 32) {
        const int64_t r = sample_index(e / a.nc, a.nr, a.M), c = sample_index(e % a.nc, a.nc, a.N);
        buf->c0[e] = (double)C[r * a.ldc + c];
    }
    if (lane == 0) buf->done = 0;
}

// One block (one warp) per sampled entry; the last block to finish reduces.
template <typename T>
__global__ void report_post_kernel(ReportArgs a) {
    const int e = blockIdx.x, lane = threadIdx.x;
    ReportBuf *buf = a.buf;
    const int64_t r = sample_index(e / a.nc, a.nr, a.M), c = sample_index(e % a.nc, a.nc, a.N);
    double p = 0.0, s = 0.0;   // this lane's part of the dot product: p + s
    for (int64_t k = lane; k < a.K; k += 32) {
        double h, rr, q;
        two_prod(op_a<T>(a, r, k), op_b<T>(a, k, c), h, rr);
        two_sum(p, h, p, q);
        s = __dadd_rn(s, __dadd_rn(q, rr));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {   // join the lanes' double-doubles
        const double p2 = __shfl_down_sync(0xffffffffu, p, o), s2 = __shfl_down_sync(0xffffffffu, s, o);
        double q;
        two_sum(p, p2, p, q);
        s = __dadd_rn(__dadd_rn(s, s2), q);
    }
    int last = 0;
    if (lane == 0) {
        const double c0 = buf->c0[e];
        double ph, pe, bh, be, out_p, q1;
        two_prod(a.alpha, p, ph, pe);
        if (a.semantics == GB_SEM_BLAS) {
            if (a.beta != 0.0) two_prod(a.beta, c0, bh, be);
            else bh = be = 0.0;
        } else if (a.semantics == GB_SEM_SCALAR_BETA) {
            bh = a.beta;
            be = 0.0;
        } else {
            two_sum(c0, a.beta, bh, be);
        }
        two_sum(ph, bh, out_p, q1);
        const double sh = __dmul_rn(a.alpha, s);
        const double ref = __dadd_rn(out_p, __dadd_rn(__dadd_rn(q1, pe), __dadd_rn(be, sh)));
        const double d = __dsub_rn((double)((const T *)a.C)[r * a.ldc + c], ref);
        buf->d2[e] = __dmul_rn(d, d);
        __threadfence();
        last = atomicAdd(&buf->done, 1u) == (unsigned)(a.nr * a.nc - 1);
    }
    if (!__shfl_sync(0xffffffffu, last, 0)) return;
    __threadfence();
    // last block: reduce the sample
    const int n = a.nr * a.nc;
    double num = 0.0, c2 = 0.0, rs = 0.0, cs = 0.0;
    for (int i = lane; i < n; i += 32) {
        num = __dadd_rn(num, ((volatile double *)buf->d2)[i]);
        c2 = __dadd_rn(c2, __dmul_rn(buf->c0[i], buf->c0[i]));
    }
    for (int i = lane; i < a.nr; i += 32) rs = __dadd_rn(rs, buf->rn2[i]);
    for (int i = lane; i < a.nc; i += 32) cs = __dadd_rn(cs, buf->cn2[i]);
    num = warp_sum(num);
    c2 = warp_sum(c2);
    rs = warp_sum(rs);
    cs = warp_sum(cs);
    if (lane == 0) {
        double den = fabs(a.alpha) * sqrt(rs) * sqrt(cs);
        if (a.semantics == GB_SEM_BLAS) {
            if (a.beta != 0.0) den += fabs(a.beta) * sqrt(c2);
        } else {
            den += fabs(a.beta) * sqrt((double)n);
            if (a.semantics == GB_SEM_ACCUM_SCALAR_BETA) den += sqrt(c2);
        }
        const double err = sqrt(num);
        *a.out = den > 0.0 ? err / den : err;
    }
}

__global__ void report_zero_kernel(double *out) { *out = 0.0; }

ReportArgs make_args(const GemmArgs &g, double *out) {
    ReportArgs a;
    a.A = g.A; a.B = g.B; a.C = g.C;
    a.lda = g.lda; a.ldb = g.ldb; a.ldc = g.ldc;
    a.M = g.M; a.N = g.N; a.K = g.K;
    a.ta = g.ta ? 1 : 0; a.tb = g.tb ? 1 : 0;
    a.nr = (int)(g.M < kS ? g.M : kS);
    a.nc = (int)(g.N < kS ? g.N : kS);
    a.semantics = g.semantics;
    a.alpha = g.alpha; a.beta = g.beta;
    a.buf = nullptr;
    a.out = out;
    return a;
}

}  // namespace

gb_status report_before(const GemmArgs &g, int bits) {
    if (g.M == 0 || g.N == 0) return ok();
    ReportArgs a = make_args(g, nullptr);
    a.buf = (ReportBuf *)aux_buffer(sizeof(ReportBuf), g.stream);
    if (!a.buf) return (gb_status)gb_get_last_status();
    if (bits == 64) report_pre_kernel<double><<<a.nr + a.nc + 1, 32, 0, g.stream>>>(a);
    else report_pre_kernel<float><<<a.nr + a.nc + 1, 32, 0, g.stream>>>(a);
    GB_LAUNCH_CHECK("report_pre_kernel");
    return ok();
}

gb_status report_after(const GemmArgs &g, int bits, double *out) {
    if (g.M == 0 || g.N == 0) {
        report_zero_kernel<<<1, 1, 0, g.stream>>>(out);
        GB_LAUNCH_CHECK("report_zero_kernel");
        return ok();
    }
    ReportArgs a = make_args(g, out);
    a.buf = (ReportBuf *)aux_buffer(sizeof(ReportBuf), g.stream);
    if (!a.buf) return (gb_status)gb_get_last_status();
    if (bits == 64) report_post_kernel<double><<<a.nr * a.nc, 32, 0, g.stream>>>(a);
    else report_post_kernel<float><<<a.nr * a.nc, 32, 0, g.stream>>>(a);
    GB_LAUNCH_CHECK("report_post_kernel");
    return ok();
}

}  // namespace gb
