// stencil.cu -- 5-point Jacobi on padded grids, with temporal blocking.
//
// Replaces stencil_vector / stencil_scalar
// (stencil_2d_V1.2/device_code/kernel_stencil.c:1042, :14): one sweep
// B = 0.2 * (N + S + E + W + C) over an (M+2) x (N+2) padded grid with a
// fixed halo.  The reference streams 128x128 (+1 halo) tiles through AM;
// here a CTA loads an output tile plus a halo of `t` cells into shared
// memory, runs `t` sweeps there (each sweep's valid region shrinks by one
// cell), and writes the final tile: HBM traffic per sweep drops to about
// (1 + halo overhead) / t of a read plus a write.  Every interior point is
// computed from the same neighbours in the same add order as the
// unblocked recurrence, so results are bit-identical for any t.
#include "gb_common.cuh"

namespace gb {
namespace {

template <typename T>
struct SOps;
template <>
struct SOps<double> {
    __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
    __device__ static double fifth() { return 0.2; }
};
template <>
struct SOps<float> {
    __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
    __device__ static float fifth() { return 0.2f; }
};

// The three reference add orders (see gbblas.h, gb_stencil_order).
template <typename T, int ORDER>
__device__ __forceinline__ T update(T top, T left, T right, T down, T mid, int64_t row) {
    using O = SOps<T>;
    if (ORDER == GB_STENCIL_HOST)
        return O::mul(O::add(O::add(O::add(O::add(top, left), right), down), mid), O::fifth());
    if (ORDER == GB_STENCIL_SCALAR)
        return O::mul(O::fifth(), O::add(O::add(O::add(O::add(top, mid), down), left), right));
    if ((row & 1) == 0) return O::mul(O::add(right, O::add(O::add(left, top), O::add(mid, down))), O::fifth());
    return O::mul(O::add(right, O::add(O::add(left, down), O::add(top, mid))), O::fifth());
}

constexpr int NT = 256;   // 32 columns x 8 row bands

// One CTA: a TH x TW output tile, loaded with a halo of `tsweeps` cells,
// `tsweeps` sweeps in shared memory, the final tile written back.  In each
// sweep warp w walks row band w of the still-valid region and lane l the
// columns l, l+32, ...; a thread keeps (top, middle, down) of its column in
// registers while it moves down the band, so a point costs three shared
// loads (down, left, right) and one store.  Cells on the grid boundary keep
// their value; cells outside the grid are computed but never read by an
// interior cell and never written back.
template <typename T, int ORDER>
__global__ void __launch_bounds__(NT) stencil_tb_kernel(const T *__restrict__ src, T *__restrict__ dst, int64_t M,
                                                        int64_t N, int tsweeps, int TH, int TW) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int H = TH + 2 * tsweeps, W = TW + 2 * tsweeps;
    T *cur = reinterpret_cast<T *>(smem_raw);
    T *nxt = cur + H * W;
    const int64_t ld = N + 2;
    const int64_t R0 = 1 + (int64_t)blockIdx.y * TH - tsweeps;   // padded coords of local (0,0)
    const int64_t C0 = 1 + (int64_t)blockIdx.x * TW - tsweeps;
    const int lane = threadIdx.x % 32, band = threadIdx.x / 32;

    for (int lr = band; lr < H; lr += NT / 32) {
        const int64_t r = R0 + lr;
        if (r < 0 || r > M + 1) continue;
        const T *srow = src + r * ld;
        for (int lc = lane; lc < W; lc += 32) {
            const int64_t c = C0 + lc;
            if (c >= 0 && c <= N + 1) cur[lr * W + lc] = srow[c];
        }
    }
    __syncthreads();

    for (int s = 1; s <= tsweeps; s++) {
        const int h = H - 2 * s;
        const int per = (h + NT / 32 - 1) / (NT / 32);
        const int rbeg = s + band * per;
        const int rend = min(rbeg + per, H - s);
        for (int lc = s + lane; lc < W - s; lc += 32) {
            if (rbeg >= rend) break;
            const int64_t gc = C0 + lc;
            const bool col_fixed = gc <= 0 || gc >= N + 1;
            const T *cp = cur + rbeg * W + lc;
            T *np = nxt + rbeg * W + lc;
            T top = cp[-W], mid = cp[0];
            int64_t gr = R0 + rbeg;
            for (int lr = rbeg; lr < rend; lr++, cp += W, np += W, gr++) {
                const T down = cp[W];
                T v = update<T, ORDER>(top, cp[-1], cp[1], down, mid, gr - 1);
                if (col_fixed || gr <= 0 || gr >= M + 1) v = mid;
                *np = v;
                top = mid;
                mid = down;
            }
        }
        __syncthreads();
        T *tmp = cur; cur = nxt; nxt = tmp;
    }

    for (int lr = tsweeps + band; lr < tsweeps + TH; lr += NT / 32) {
        const int64_t r = R0 + lr;
        if (r < 1 || r > M) continue;
        T *drow = dst + r * ld;
        for (int lc = tsweeps + lane; lc < tsweeps + TW; lc += 32) {
            const int64_t c = C0 + lc;
            if (c >= 1 && c <= N) drow[c] = cur[lr * W + lc];
        }
    }
}

// FP32 form, no shared memory: register-streamed temporal blocking.  A warp
// owns a strip of 128 columns (lane l: columns 4l .. 4l+3) and walks a
// segment of rows top to bottom, one input row per step.  Sweep level
// l = 1..T keeps the last two rows of level l-1 in registers; when level l-1
// produces row rho+1, level l computes row rho from (rho-1, rho, rho+1)
// with the left / right neighbours of the middle row from the adjacent
// lanes (two shuffles per four points).  The level-T rows are written out.
// Each level loses one column at each strip edge and one row at each
// segment end, so a strip writes 128 - 2T columns and a segment reads T
// rows of halo above and below.  Every point gets the same neighbours in the
// same add order as one sweep at a time, so results are bit-identical.
constexpr int RS_W = 128, RS_SEG = 256, RS_NT = 256;

template <typename E, int T, int ORDER>
__global__ void __launch_bounds__(RS_NT) stencil_rs_kernel(const E *__restrict__ src, E *__restrict__ dst,
                                                           int64_t M, int64_t N, int strips, int segs) {
    const int lane = threadIdx.x % 32;
    const int64_t wid = (int64_t)blockIdx.x * (RS_NT / 32) + threadIdx.x / 32;
    if (wid >= (int64_t)strips * segs) return;   // whole warp
    const int sx = (int)(wid % strips), sy = (int)(wid / strips);
    const int64_t ld = N + 2;
    const int64_t c0 = 1 + (int64_t)sx * (RS_W - 2 * T) - T;   // padded column of lane 0, q = 0
    const int64_t out_r0 = 1 + (int64_t)sy * RS_SEG;            // padded rows written: [out_r0, out_r1)
    const int64_t out_r1 = out_r0 + RS_SEG < M + 1 ? out_r0 + RS_SEG : M + 1;
    const int64_t cl = c0 + 4 * lane;                            // this lane's first column

    bool cfix[4], cload[4], cstore[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int64_t gc = cl + q;
        const int lc = 4 * lane + q;
        cfix[q] = gc <= 0 || gc >= N + 1;
        cload[q] = gc >= 0 && gc <= N + 1;
        cstore[q] = lc >= T && lc < RS_W - T && gc >= 1 && gc <= N;
    }

    E p2[T][4], p1[T][4];   // level l-1 rows rho-1 and rho of level l's window
#pragma unroll
    for (int l = 0; l < T; l++)
#pragma unroll
        for (int q = 0; q < 4; q++) p2[l][q] = p1[l][q] = E(0);

    for (int64_t i = out_r0 - T - 1; i < out_r1 + T; i++) {   // input row i (level 0)
        E x[4] = {E(0), E(0), E(0), E(0)};
        if (i >= 0 && i <= M + 1) {
            const E *row = src + i * ld + cl;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (cload[q]) x[q] = __ldg(row + q);
        }
#pragma unroll
        for (int l = 0; l < T; l++) {
            // level l+1, row rho = i - l - 1: top p2[l], middle p1[l], down x
            const int64_t gr = i - l - 1;
            const E left0 = __shfl_up_sync(0xffffffffu, p1[l][3], 1);
            const E right3 = __shfl_down_sync(0xffffffffu, p1[l][0], 1);
            const bool rfix = gr <= 0 || gr >= M + 1;
            E v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const E lft = q == 0 ? left0 : p1[l][q - 1];
                const E rgt = q == 3 ? right3 : p1[l][q + 1];
                v[q] = (rfix || cfix[q]) ? p1[l][q] : update<E, ORDER>(p2[l][q], lft, rgt, x[q], p1[l][q], gr - 1);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                p2[l][q] = p1[l][q];
                p1[l][q] = x[q];
                x[q] = v[q];
            }
        }
        // x: level T, row i - T
        const int64_t ro = i - T;
        if (ro >= out_r0 && ro < out_r1) {
            E *row = dst + ro * ld + cl;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (cstore[q]) row[q] = x[q];
        }
    }
}

template <typename E, int T>
void launch_rs(const E *src, E *dst, int64_t M, int64_t N, int order, cudaStream_t st) {
    const int strips = (int)ceil_div(N, RS_W - 2 * T);
    const int segs = (int)ceil_div(M, RS_SEG);
    const unsigned blocks = (unsigned)ceil_div((int64_t)strips * segs, RS_NT / 32);
    if (order == 0) stencil_rs_kernel<E, T, 0><<<blocks, RS_NT, 0, st>>>(src, dst, M, N, strips, segs);
    else if (order == 1) stencil_rs_kernel<E, T, 1><<<blocks, RS_NT, 0, st>>>(src, dst, M, N, strips, segs);
    else stencil_rs_kernel<E, T, 2><<<blocks, RS_NT, 0, st>>>(src, dst, M, N, strips, segs);
}

// 9-point stencil with a 3x3 weight window (w[0..2] the row above, w[3..5]
// the row, w[6..8] the row below): r = w0*a_tl, then eight fused
// multiply-adds in window order.  Same register-streaming scheme as the
// 5-point kernel; every row that enters a level's window brings the left /
// right neighbours of its edge columns (two shuffles per row and level).
template <typename E>
struct W9 {
    E w[9];
};

template <typename E>
struct Row4 {
    E v[4];
    E lft, rgt;   // column 4*lane - 1 and 4*lane + 4
};

template <typename E>
__device__ __forceinline__ E fma_rn(E a, E b, E c);
template <>
__device__ __forceinline__ float fma_rn<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ double fma_rn<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename E>
__device__ __forceinline__ E mul_rn(E a, E b);
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }

template <typename E, int T>
__global__ void __launch_bounds__(RS_NT) stencil9_rs_kernel(const E *__restrict__ src, E *__restrict__ dst,
                                                            int64_t M, int64_t N, int strips, int segs, W9<E> w) {
    const int lane = threadIdx.x % 32;
    const int64_t wid = (int64_t)blockIdx.x * (RS_NT / 32) + threadIdx.x / 32;
    if (wid >= (int64_t)strips * segs) return;   // whole warp
    const int sx = (int)(wid % strips), sy = (int)(wid / strips);
    const int64_t ld = N + 2;
    const int64_t c0 = 1 + (int64_t)sx * (RS_W - 2 * T) - T;
    const int64_t out_r0 = 1 + (int64_t)sy * RS_SEG;
    const int64_t out_r1 = out_r0 + RS_SEG < M + 1 ? out_r0 + RS_SEG : M + 1;
    const int64_t cl = c0 + 4 * lane;

    bool cfix[4], cload[4], cstore[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int64_t gc = cl + q;
        const int lc = 4 * lane + q;
        cfix[q] = gc <= 0 || gc >= N + 1;
        cload[q] = gc >= 0 && gc <= N + 1;
        cstore[q] = lc >= T && lc < RS_W - T && gc >= 1 && gc <= N;
    }

    Row4<E> p2[T], p1[T];
#pragma unroll
    for (int l = 0; l < T; l++) {
#pragma unroll
        for (int q = 0; q < 4; q++) p2[l].v[q] = p1[l].v[q] = E(0);
        p2[l].lft = p2[l].rgt = p1[l].lft = p1[l].rgt = E(0);
    }

    for (int64_t i = out_r0 - T - 1; i < out_r1 + T; i++) {
        Row4<E> x;
#pragma unroll
        for (int q = 0; q < 4; q++) x.v[q] = E(0);
        if (i >= 0 && i <= M + 1) {
            const E *row = src + i * ld + cl;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (cload[q]) x.v[q] = __ldg(row + q);
        }
#pragma unroll
        for (int l = 0; l < T; l++) {
            x.lft = __shfl_up_sync(0xffffffffu, x.v[3], 1);
            x.rgt = __shfl_down_sync(0xffffffffu, x.v[0], 1);
            const int64_t gr = i - l - 1;
            const bool rfix = gr <= 0 || gr >= M + 1;
            const Row4<E> &t = p2[l], &m = p1[l];
            Row4<E> v;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const E tl = q == 0 ? t.lft : t.v[q - 1], tr = q == 3 ? t.rgt : t.v[q + 1];
                const E ml = q == 0 ? m.lft : m.v[q - 1], mr = q == 3 ? m.rgt : m.v[q + 1];
                const E dl = q == 0 ? x.lft : x.v[q - 1], dr = q == 3 ? x.rgt : x.v[q + 1];
                E r = mul_rn(w.w[0], tl);
                r = fma_rn(w.w[1], t.v[q], r);
                r = fma_rn(w.w[2], tr, r);
                r = fma_rn(w.w[3], ml, r);
                r = fma_rn(w.w[4], m.v[q], r);
                r = fma_rn(w.w[5], mr, r);
                r = fma_rn(w.w[6], dl, r);
                r = fma_rn(w.w[7], x.v[q], r);
                r = fma_rn(w.w[8], dr, r);
                v.v[q] = (rfix || cfix[q]) ? m.v[q] : r;
            }
            p2[l] = p1[l];
            p1[l] = x;
            x = v;
        }
        const int64_t ro = i - T;
        if (ro >= out_r0 && ro < out_r1) {
            E *row = dst + ro * ld + cl;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (cstore[q]) row[q] = x.v[q];
        }
    }
}

template <typename E, int T>
void launch_rs9(const E *src, E *dst, int64_t M, int64_t N, const W9<E> &w, cudaStream_t st) {
    const int strips = (int)ceil_div(N, RS_W - 2 * T);
    const int segs = (int)ceil_div(M, RS_SEG);
    const unsigned blocks = (unsigned)ceil_div((int64_t)strips * segs, RS_NT / 32);
    stencil9_rs_kernel<E, T><<<blocks, RS_NT, 0, st>>>(src, dst, M, N, strips, segs, w);
}

template <typename E>
gb_status stencil9(int64_t M, int64_t N, E *A, E *B, int iters, const E *w_host, void *stream) {
    GB_CHECK_ARG(M >= 0 && N >= 0, "stencil9: negative size");
    GB_CHECK_ARG(iters >= 0, "stencil9: negative iteration count");
    if (M == 0 || N == 0 || iters == 0) return ok();
    GB_CHECK_ARG(A && B && A != B, "stencil9: A and B must be distinct device buffers");
    GB_CHECK_ARG(w_host != nullptr, "stencil9: null weight window");
    GB_CHECK_ARG((M + RS_SEG - 1) / RS_SEG < (1 << 30), "stencil9: M too large");
    W9<E> w;
    for (int i = 0; i < 9; i++) w.w[i] = w_host[i];
    // FP32: 4 sweeps per pass (the window rows of 4 levels fill the register
    // budget); FP64 is bound by the FP64 pipe: one sweep per pass
    const int tmax = sizeof(E) == 4 ? 4 : 1;
    int L = (int)ceil_div(iters, tmax);
    if ((L & 1) != (iters & 1)) L += 1;   // result in B for odd iters, in A for even
    cudaStream_t st = as_stream(stream);
    int done = 0;
    for (int l = 0; l < L; l++) {
        int t = (iters - done) / (L - l);
        if ((iters - done) % (L - l)) t += 1;
        const E *src = (l % 2 == 0) ? A : B;
        E *dst = (l % 2 == 0) ? B : A;
        switch (t) {
            case 1: launch_rs9<E, 1>(src, dst, M, N, w, st); break;
            case 2: launch_rs9<E, (sizeof(E) == 4 ? 2 : 1)>(src, dst, M, N, w, st); break;
            case 3: launch_rs9<E, (sizeof(E) == 4 ? 3 : 1)>(src, dst, M, N, w, st); break;
            default: launch_rs9<E, (sizeof(E) == 4 ? 4 : 1)>(src, dst, M, N, w, st); break;
        }
        GB_LAUNCH_CHECK("stencil9_rs_kernel");
        done += t;
    }
    return ok();
}

template <typename T>
gb_status stencil(int64_t M, int64_t N, T *A, T *B, int iters, int order, void *stream) {
    GB_CHECK_ARG(M >= 0 && N >= 0, "stencil2d: negative size");
    GB_CHECK_ARG(iters >= 0, "stencil2d: negative iteration count");
    GB_CHECK_ARG(order >= 0 && order <= 2, "stencil2d: order %d not in 0..2", order);
    if (M == 0 || N == 0 || iters == 0) return ok();
    GB_CHECK_ARG(A && B && A != B, "stencil2d: A and B must be distinct device buffers");
    // tile and temporal depth: FP32 is HBM-bound (block 8 sweeps); FP64 is
    // bound by the FP64 pipe, where recomputing halos only costs, so t = 1.
    const char *rsenv = getenv("GB_STENCIL_RS");   // "0": the shared-memory kernel (measurement)
    // FP64 keeps the shared-memory kernel with t = 1: it is bound by the FP64
    // pipe, and the streaming form measured slower there (1.38 vs 1.64 TB/s)
    const bool rs = sizeof(T) == 4 && !(rsenv && rsenv[0] == '0');
    const int tmax = sizeof(T) == 4 ? 8 : 1;
    const int TH = sizeof(T) == 4 ? 64 : 32, TW = sizeof(T) == 4 ? 128 : 64;
    // launches L with L == iters (mod 2) so the result lands in B for odd
    // iters and in A for even iters, as with one sweep per launch
    int L = (int)ceil_div(iters, tmax);
    if ((L & 1) != (iters & 1)) L += 1;
    dim3 grid((unsigned)ceil_div(N, TW), (unsigned)ceil_div(M, TH));
    GB_CHECK_ARG(grid.y <= 65535u, "stencil2d: M too large");
    cudaStream_t st = as_stream(stream);
    int done = 0;
    for (int l = 0; l < L; l++) {
        int t = (iters - done) / (L - l);      // spread evenly
        int rem = (iters - done) % (L - l);
        if (rem) t += 1;
        const T *src = (l % 2 == 0) ? A : B;
        T *dst = (l % 2 == 0) ? B : A;
        if (rs) {
            {
                const float *s4 = (const float *)src;
                float *d4 = (float *)dst;
                switch (t) {
                    case 1: launch_rs<float, 1>(s4, d4, M, N, order, st); break;
                    case 2: launch_rs<float, 2>(s4, d4, M, N, order, st); break;
                    case 3: launch_rs<float, 3>(s4, d4, M, N, order, st); break;
                    case 4: launch_rs<float, 4>(s4, d4, M, N, order, st); break;
                    case 5: launch_rs<float, 5>(s4, d4, M, N, order, st); break;
                    case 6: launch_rs<float, 6>(s4, d4, M, N, order, st); break;
                    case 7: launch_rs<float, 7>(s4, d4, M, N, order, st); break;
                    default: launch_rs<float, 8>(s4, d4, M, N, order, st); break;
                }
            }
            GB_LAUNCH_CHECK("stencil_rs_kernel");
            done += t;
            continue;
        }
        size_t smem = 2 * (size_t)(TH + 2 * t) * (TW + 2 * t) * sizeof(T);
        switch (order) {
            case 0:
                cudaFuncSetAttribute(stencil_tb_kernel<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                stencil_tb_kernel<T, 0><<<grid, NT, smem, st>>>(src, dst, M, N, t, TH, TW);
                break;
            case 1:
                cudaFuncSetAttribute(stencil_tb_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                stencil_tb_kernel<T, 1><<<grid, NT, smem, st>>>(src, dst, M, N, t, TH, TW);
                break;
            default:
                cudaFuncSetAttribute(stencil_tb_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                stencil_tb_kernel<T, 2><<<grid, NT, smem, st>>>(src, dst, M, N, t, TH, TW);
                break;
        }
        GB_LAUNCH_CHECK("stencil_tb_kernel");
        done += t;
    }
    return ok();
}

}  // namespace
}  // namespace gb

extern "C" {

gb_status gb_stencil2d_f64(int64_t M, int64_t N, double *A, double *B, int iters, int order, void *stream) {
    return gb::stencil<double>(M, N, A, B, iters, order, stream);
}

gb_status gb_stencil2d_f32(int64_t M, int64_t N, float *A, float *B, int iters, int order, void *stream) {
    return gb::stencil<float>(M, N, A, B, iters, order, stream);
}

gb_status gb_stencil9_f32(int64_t M, int64_t N, float *A, float *B, int iters, const float *w, void *stream) {
    return gb::stencil9<float>(M, N, A, B, iters, w, stream);
}

gb_status gb_stencil9_f64(int64_t M, int64_t N, double *A, double *B, int iters, const double *w, void *stream) {
    return gb::stencil9<double>(M, N, A, B, iters, w, stream);
}

}  // extern "C"
