// serve.cu -- request loop: HBM-budget admission, continuous batching into
// grouped launches, CUDA-graph replay, per-request latency (p50 / p99).
//
// The reference host runs one kernel at a time (hthread_group_exec +
// hthread_group_wait, sgemm_release_V1.3.2/host_code/sgemm_demo.c:144-145);
// this is the GB300 serving layer built on the same hot-path kernels.  It has
// no reference counterpart.
//
// Requests (GEMM, transpose, Jacobi) carry device pointers to operands the
// caller keeps resident.  A request is charged the bytes of its operands
// while it is in flight; it is admitted when the in-flight total plus its
// charge fits the budget (FIFO; a request larger than the whole budget is
// rejected).  A dispatcher thread takes every admitted request as soon as it
// is admitted: GEMMs below the grouping threshold go together into one launch
// of the grouped persistent kernel (replayed from a CUDA graph per slot),
// the rest go one launch each with the algorithm the autotune table (or the
// AUTO heuristic) picks, round-robin over the stream pool.  A host callback
// on the stream stamps completion, releases the charge and wakes the
// dispatcher, so new requests are admitted while earlier ones run.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <tuple>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace gb {

static double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// ------------------------------------------------------------ autotune table
namespace {
struct TuneKey {
    int bits, ta, tb, lm, ln, lk;
    bool operator<(const TuneKey &o) const {
        return std::tie(bits, ta, tb, lm, ln, lk) < std::tie(o.bits, o.ta, o.tb, o.lm, o.ln, o.lk);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, gb_tune_choice> g_tune;

int lg(int64_t x) {   // bucket: round(log2(x)) (0 for x <= 1)
    if (x <= 1) return 0;
    return (int)lround(log2((double)x));
}

TuneKey key_of(int bits, bool ta, bool tb, int64_t M, int64_t N, int64_t K) {
    return TuneKey{bits, ta ? 1 : 0, tb ? 1 : 0, lg(M), lg(N), lg(K)};
}
}  // namespace

bool tuned_choice(int bits, bool ta, bool tb, int64_t M, int64_t N, int64_t K, gb_tune_choice *out) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key_of(bits, ta, tb, M, N, K));
    if (it == g_tune.end()) return false;
    *out = it->second;
    return true;
}

// ------------------------------------------------------------------- server
namespace {

struct Pending {
    gb_request r;
    uint64_t bytes;
    double t_submit;
};

struct Batch;   // completion context of one launch

// Bucket of a one-launch request's graph: requests of one bucket usually launch the same kernels,
// so the cached executable graph is updated in place (cudaGraphExecUpdate) instead of rebuilt.
struct GKey {
    int op, bits, ta, tb, algo, lm, ln, lk, li;
    bool operator<(const GKey &o) const {
        return std::tie(op, bits, ta, tb, algo, lm, ln, lk, li) <
               std::tie(o.op, o.bits, o.ta, o.tb, o.algo, o.lm, o.ln, o.lk, o.li);
    }
};

}  // namespace

struct Server {
    gb_server_config cfg;
    std::mutex mu;
    std::condition_variable cv_dispatch, cv_done;
    std::deque<Pending> waiting;
    uint64_t inflight_bytes = 0;
    int64_t inflight = 0, submitted = 0, completed = 0, rejected = 0, failed = 0;
    int64_t launches = 0, grouped_launches = 0, grouped_requests = 0;
    double t_first = 0, t_last = 0;
    std::vector<double> latencies;
    std::vector<uint64_t> done_tags;
    std::vector<double> done_lat;
    std::vector<cudaStream_t> streams;
    std::vector<size_t> ws_reserved;                          // workspace reserved per stream
    std::vector<std::map<GKey, cudaGraphExec_t>> execs;       // one-launch graphs per stream
    std::set<GKey> seen;                                      // buckets that ran once without a graph
    std::atomic<int64_t> graph_launches{0}, graph_instantiations{0};
    int64_t urgent_launches = 0;   // launches on the high-priority streams (under mu)
    size_t rr = 0, rr_short = 0;
    GroupRunner *grouped = nullptr;
    std::thread dispatcher;
    bool stop = false;
    int device = 0;
    int last_error = GB_OK;
};

namespace {

struct Batch {
    Server *s;
    std::vector<std::pair<uint64_t, double>> reqs;   // tag, submit time
    uint64_t bytes;
};

void CUDART_CB on_done(void *p) {
    Batch *b = static_cast<Batch *>(p);
    Server *s = b->s;
    const double t = now_s();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &q : b->reqs) {
            const double lat = t - q.second;
            s->latencies.push_back(lat);
            s->done_tags.push_back(q.first);
            s->done_lat.push_back(lat);
        }
        s->completed += (int64_t)b->reqs.size();
        s->inflight -= (int64_t)b->reqs.size();
        s->inflight_bytes -= b->bytes;
        s->t_last = t;
    }
    s->cv_dispatch.notify_all();
    s->cv_done.notify_all();
    delete b;
}

uint64_t request_bytes(const gb_request &r) {
    const uint64_t es = r.dtype_bits == 64 ? 8 : 4;
    if (r.bytes) return r.bytes;
    switch (r.op) {
        case GB_OP_GEMM: {
            const uint64_t a = (uint64_t)r.M * r.K, b = (uint64_t)r.K * r.N, c = (uint64_t)r.M * r.N;
            return es * (a + b + c);
        }
        case GB_OP_TRANSPOSE: return es * 2 * (uint64_t)r.M * r.N;
        default: return es * 2 * (uint64_t)(r.M + 2) * (r.N + 2);
    }
}

gb_status validate(const gb_request &r) {
    GB_CHECK_ARG(r.op >= GB_OP_GEMM && r.op <= GB_OP_STENCIL, "server: unknown op %d", r.op);
    GB_CHECK_ARG(r.dtype_bits == 32 || r.dtype_bits == 64, "server: dtype_bits must be 32 or 64");
    GB_CHECK_ARG(r.M >= 0 && r.N >= 0 && r.K >= 0, "server: negative dimension");
    if (r.op == GB_OP_GEMM) {
        gb_gemm_desc d;
        memset(&d, 0, sizeof(d));
        d.dtype_bits = r.dtype_bits; d.transA = r.transA; d.transB = r.transB; d.semantics = r.semantics;
        d.M = r.M; d.N = r.N; d.K = r.K; d.A = r.A; d.lda = r.lda; d.B = r.B; d.ldb = r.ldb; d.C = r.C; d.ldc = r.ldc;
        return check_desc(d, 0);
    }
    if (r.op == GB_OP_TRANSPOSE) {
        GB_CHECK_ARG(r.lda >= r.N && r.ldb >= r.M, "server: transpose leading dimensions");
        GB_CHECK_ARG((r.M == 0 || r.N == 0) || (r.A && r.B && r.A != r.B), "server: transpose pointers");
    } else {
        GB_CHECK_ARG(r.iters >= 0 && r.order >= 0 && r.order <= 2, "server: stencil iters/order");
        GB_CHECK_ARG((r.M == 0 || r.N == 0) || (r.A && r.C && (const void *)r.A != r.C), "server: stencil pointers");
    }
    return ok();
}

bool groupable(const Server *s, const gb_request &r) {
    if (!s->cfg.use_grouped || r.op != GB_OP_GEMM || r.algo != GB_ALGO_AUTO) return false;
    const double work = (double)r.M * r.N * r.K;
    const int64_t small = r.M < r.N ? r.M : r.N;
    if (small <= 64) return false;   // the skinny kernel streams those better
    return work <= s->cfg.group_max_work;
}

gb_status launch_one(Server *s, const gb_request &r, cudaStream_t st) {
    if (r.op == GB_OP_GEMM) {
        gb_gemm_opts o;
        gb_gemm_opts_init(&o);
        o.stream = st;
        o.semantics = r.semantics;
        o.algo = r.algo;
        gb_tune_choice t;
        if (o.algo == GB_ALGO_AUTO && tuned_choice(r.dtype_bits, is_trans(r.transA), is_trans(r.transB), r.M, r.N,
                                                   r.K, &t)) {
            o.algo = t.algo;
            o.accum_k = t.accum_k;
            o.split_k = t.split_k;
            o.ozaki_slices = t.ozaki_slices;
        }
        if (r.dtype_bits == 64)
            return gb_dgemm(r.transA, r.transB, r.M, r.N, r.K, r.alpha, (const double *)r.A, r.lda,
                            (const double *)r.B, r.ldb, r.beta, (double *)r.C, r.ldc, &o);
        return gb_sgemm(r.transA, r.transB, r.M, r.N, r.K, (float)r.alpha, (const float *)r.A, r.lda,
                        (const float *)r.B, r.ldb, (float)r.beta, (float *)r.C, r.ldc, &o);
    }
    if (r.op == GB_OP_TRANSPOSE) {
        if (r.dtype_bits == 64)
            return gb_transpose_f64(r.M, r.N, (const double *)r.A, r.lda, (double *)r.B, r.ldb, st);
        return gb_transpose_f32(r.M, r.N, (const float *)r.A, r.lda, (float *)r.B, r.ldb, st);
    }
    (void)s;
    if (r.dtype_bits == 64)
        return gb_stencil2d_f64(r.M, r.N, (double *)r.A, (double *)r.C, r.iters, r.order, st);
    return gb_stencil2d_f32(r.M, r.N, (float *)r.A, (float *)r.C, r.iters, r.order, st);
}

// A one-launch request through a CUDA graph: its launches are captured on the stream (after the
// stream's workspace has been grown to the request's bound, since a capture cannot allocate) and
// replayed by the bucket's executable graph, updated in place when the launches match.  Anything
// that cannot be captured runs as plain launches.
gb_status launch_request(Server *s, const gb_request &r, size_t si, bool *graphed) {
    cudaStream_t st = s->streams[si];
    *graphed = false;
    if (!s->cfg.use_graphs) return launch_one(s, r, st);
    int algo = r.algo, slices = 0, split_k = 0;
    const bool ta = is_trans(r.transA), tb = is_trans(r.transB);
    if (r.op == GB_OP_GEMM) {
        gb_tune_choice t;
        if (algo == GB_ALGO_AUTO && tuned_choice(r.dtype_bits, ta, tb, r.M, r.N, r.K, &t)) {
            algo = t.algo;
            slices = t.ozaki_slices;
            split_k = t.split_k;
        }
        algo = resolve_algo(r.dtype_bits, algo, ta, tb, r.M, r.N, r.K);
    }
    const GKey key{r.op, r.dtype_bits, ta ? 1 : 0, tb ? 1 : 0, algo, lg(r.M), lg(r.N), lg(r.K), lg(r.iters)};
    // The first request of a bucket runs as plain launches: it loads the kernels and sets their
    // attributes outside any capture, and a shape seen once builds no graph.
    if (s->seen.insert(key).second) return launch_one(s, r, st);
    const size_t need =
        r.op == GB_OP_GEMM ? gemm_workspace_bound(r.dtype_bits, algo, ta, tb, r.M, r.N, r.K, r.A, r.lda, r.B, r.ldb,
                                                  slices, split_k)
                           : 0;
    if (need > s->ws_reserved[si]) {
        const size_t want = std::max(need, 2 * s->ws_reserved[si]);
        if (gb_workspace_reserve(want, st) != GB_OK) {
            gb_clear_last_status();
            return launch_one(s, r, st);
        }
        s->ws_reserved[si] = want;
    }
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return launch_one(s, r, st);
    }
    const gb_status rc = launch_one(s, r, st);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (rc != GB_OK || ce != cudaSuccess || g == nullptr) {   // not capturable: plain launches
        cudaGetLastError();
        gb_clear_last_status();
        if (g) cudaGraphDestroy(g);
        return launch_one(s, r, st);
    }
    auto &cache = s->execs[si];
    cudaGraphExec_t ex = nullptr;
    auto it = cache.find(key);
    if (it != cache.end()) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(it->second, g, &info) == cudaSuccess) {
            ex = it->second;
        } else {   // other launches than the cached graph's: build a new one
            cudaGetLastError();
            cudaGraphExecDestroy(it->second);
            cache.erase(it);
        }
    }
    if (!ex) {
        if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphDestroy(g);
            return launch_one(s, r, st);
        }
        cache[key] = ex;
        s->graph_instantiations++;
    }
    cudaGraphDestroy(g);
    const cudaError_t le = cudaGraphLaunch(ex, st);
    if (le != cudaSuccess) return cuda_status(le, "server: cudaGraphLaunch");
    *graphed = true;
    s->graph_launches++;
    return GB_OK;
}

// A request's duration at the rates the library reaches on GB300 (tensor-core GEMM forms ~300
// TFLOP/s FP32 and ~35 FP64, HBM-bound streams ~5 TB/s), in microseconds: only to tell short
// requests from long ones.
double estimate_us(const gb_request &r) {
    const double es = r.dtype_bits == 64 ? 8.0 : 4.0;
    const double M = (double)r.M, N = (double)r.N, K = (double)r.K;
    if (r.op == GB_OP_GEMM) {
        const double flops = 2.0 * M * N * K;
        const double bytes = es * (M * K + K * N + 2.0 * M * N);
        return std::max(flops / (r.dtype_bits == 64 ? 35e6 : 300e6), bytes / 5e6) + 5.0;
    }
    if (r.op == GB_OP_TRANSPOSE) return 2.0 * es * M * N / 5e6 + 5.0;
    return 2.0 * es * M * N * (double)std::max(r.iters, 1) / 8e6 + 5.0;   // Jacobi sweeps
}

// Streams 0..short_streams-1 carry the short requests when priorities are on.
bool urgent_stream(const Server *s, size_t si) {
    return s->streams.size() >= 2 && s->cfg.short_us > 0 && si < (size_t)s->cfg.short_streams;
}

// Short requests round-robin over the high-priority streams 0..h-1, the rest over h..n-1 (every
// stream in turn when there is one stream or priorities are off).
size_t pick_stream(Server *s, double est_us) {
    const size_t n = s->streams.size();
    if (n < 2 || s->cfg.short_us <= 0) return s->rr++ % n;
    const size_t h = (size_t)s->cfg.short_streams;
    if (est_us < s->cfg.short_us) return s->rr_short++ % h;
    return h + (s->rr++ % (n - h));
}

void dispatcher_main(Server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_dispatch.wait(lk, [s] {
            return s->stop || (!s->waiting.empty() &&
                               s->inflight_bytes + s->waiting.front().bytes <= s->cfg.hbm_budget_bytes &&
                               s->inflight < s->cfg.max_inflight);
        });
        if (s->stop && s->waiting.empty()) break;
        if (s->stop && s->inflight_bytes + s->waiting.front().bytes > s->cfg.hbm_budget_bytes) {
            s->cv_dispatch.wait(lk);
            continue;
        }
        // admit FIFO while the budget allows
        std::vector<Pending> admitted;
        while (!s->waiting.empty() && s->inflight_bytes + s->waiting.front().bytes <= s->cfg.hbm_budget_bytes &&
               s->inflight < s->cfg.max_inflight) {
            admitted.push_back(s->waiting.front());
            s->inflight_bytes += s->waiting.front().bytes;
            s->inflight++;
            s->waiting.pop_front();
        }
        lk.unlock();

        std::vector<gb_gemm_desc> group;
        std::vector<Pending> group_reqs;
        for (auto &p : admitted) {
            if (groupable(s, p.r) && (int)group.size() < s->cfg.max_batch) {
                gb_gemm_desc d;
                memset(&d, 0, sizeof(d));
                d.dtype_bits = p.r.dtype_bits; d.transA = p.r.transA; d.transB = p.r.transB;
                d.semantics = p.r.semantics; d.M = p.r.M; d.N = p.r.N; d.K = p.r.K;
                d.alpha = p.r.alpha; d.beta = p.r.beta;
                d.A = p.r.A; d.lda = p.r.lda; d.B = p.r.B; d.ldb = p.r.ldb; d.C = p.r.C; d.ldc = p.r.ldc;
                group.push_back(d);
                group_reqs.push_back(p);
                continue;
            }
            const double est = estimate_us(p.r);
            const size_t si = pick_stream(s, est);
            // a long request on the normal streams plans for a share of the SMs only
            const bool capped = s->cfg.long_sm_percent < 100 && s->cfg.short_us > 0 && est >= s->cfg.short_us &&
                                s->streams.size() >= 2 && !s->cfg.dry_run;
            if (capped) {
                set_sm_cap(0);
                set_sm_cap((int)((int64_t)sm_count() * s->cfg.long_sm_percent / 100));
            }
            cudaStream_t st = s->streams[si];
            Batch *b = new Batch{s, {{p.r.tag, p.t_submit}}, p.bytes};
            bool graphed = false;
            gb_status rc = s->cfg.dry_run ? GB_OK : launch_request(s, p.r, si, &graphed);
            if (capped) set_sm_cap(0);
            if (rc != GB_OK) {
                std::lock_guard<std::mutex> g(s->mu);
                s->failed++;
                s->last_error = rc;
            }
            if (s->cfg.dry_run) on_done(b);
            else cudaLaunchHostFunc(st, on_done, b);
            std::lock_guard<std::mutex> g(s->mu);
            s->launches++;
            if (urgent_stream(s, si)) s->urgent_launches++;
        }
        if (!group.empty()) {
            const size_t gsi = pick_stream(s, 0.0);   // grouped launches are short
            cudaStream_t st = s->streams[gsi];
            Batch *b = new Batch{s, {}, 0};
            for (auto &p : group_reqs) {
                b->reqs.push_back({p.r.tag, p.t_submit});
                b->bytes += p.bytes;
            }
            gb_status rc = s->cfg.dry_run ? GB_OK
                                          : group_runner_run(s->grouped, group.data(), (int)group.size(), st,
                                                             s->cfg.use_graphs);
            if (rc != GB_OK) {
                std::lock_guard<std::mutex> g(s->mu);
                s->failed += (int64_t)group.size();
                s->last_error = rc;
            }
            if (s->cfg.dry_run) on_done(b);
            else cudaLaunchHostFunc(st, on_done, b);
            std::lock_guard<std::mutex> g(s->mu);
            s->launches++;
            if (urgent_stream(s, gsi)) s->urgent_launches++;
            if (rc == GB_OK && s->cfg.use_graphs && !s->cfg.dry_run) s->graph_launches++;
            s->grouped_launches++;
            s->grouped_requests += (int64_t)group.size();
        }
        lk.lock();
    }
}

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    double pos = q * (v.size() - 1);
    size_t i = (size_t)pos;
    double f = pos - i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace
}  // namespace gb

using gb::Server;

extern "C" {

void gb_server_config_init(gb_server_config *c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->hbm_budget_bytes = 48ull << 30;
    c->streams = 6;
    c->max_batch = 256;
    c->max_inflight = 1 << 20;
    c->use_graphs = 1;
    c->use_grouped = 1;
    c->group_max_work = 512.0 * 512.0 * 512.0;
    c->short_us = 200.0;
    c->short_streams = 2;
    c->long_sm_percent = 100;
}

gb_status gb_server_create(const gb_server_config *cfg, gb_server **out) {
    GB_CHECK_ARG(out != nullptr, "gb_server_create: null out-pointer");
    *out = nullptr;
    gb_server_config c;
    if (cfg) c = *cfg; else gb_server_config_init(&c);
    GB_CHECK_ARG(c.hbm_budget_bytes > 0, "gb_server_create: zero HBM budget");
    GB_CHECK_ARG(c.streams >= 1 && c.streams <= 64, "gb_server_create: streams must be 1..64");
    GB_CHECK_ARG(c.max_batch >= 1 && c.max_batch <= 4096, "gb_server_create: max_batch must be 1..4096");
    GB_CHECK_ARG(c.max_inflight >= 1, "gb_server_create: max_inflight must be positive");
    GB_CHECK_ARG(c.short_us <= 0 || c.short_streams >= 1, "gb_server_create: short_streams must be positive");
    if (c.short_streams >= c.streams) c.short_streams = c.streams - 1;   // at least one stream for long work
    GB_CHECK_ARG(c.long_sm_percent >= 1 && c.long_sm_percent <= 100, "gb_server_create: long_sm_percent must be 1..100");
    Server *s = new Server();
    s->cfg = c;
    if (!c.dry_run) {
        cudaGetDevice(&s->device);
        for (int i = 0; i < c.streams; i++) {
            // stream 0 carries the short requests at the device's highest priority (when there
            // are at least two streams and short_us > 0)
            int lo = 0, hi = 0;
            cudaDeviceGetStreamPriorityRange(&lo, &hi);
            const bool urgent = i < c.short_streams && c.streams >= 2 && c.short_us > 0;
            cudaStream_t st;
            cudaError_t e = cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, urgent ? hi : lo);
            if (e != cudaSuccess) {
                for (auto x : s->streams) cudaStreamDestroy(x);
                delete s;
                return gb::cuda_status(e, "gb_server_create: stream");
            }
            s->streams.push_back(st);
            s->ws_reserved.push_back(c.workspace_bytes);
            s->execs.emplace_back();
            if (c.workspace_bytes) {
                gb_status r = gb_workspace_reserve(c.workspace_bytes, st);
                if (r != GB_OK) {
                    for (auto x : s->streams) cudaStreamDestroy(x);
                    delete s;
                    return r;
                }
            }
        }
        s->grouped = gb::group_runner_create(2 * c.streams, c.max_batch);
    } else {   // no device work: the streams are placeholders, so that routing runs as it would
        for (int i = 0; i < c.streams; i++) {
            s->streams.push_back(nullptr);
            s->ws_reserved.push_back(0);
            s->execs.emplace_back();
        }
    }
    s->dispatcher = std::thread(gb::dispatcher_main, s);
    *out = reinterpret_cast<gb_server *>(s);
    return gb::ok();
}

gb_status gb_server_submit(gb_server *sv, const gb_request *req) {
    GB_CHECK_ARG(sv && req, "gb_server_submit: null argument");
    Server *s = reinterpret_cast<Server *>(sv);
    gb_status v = gb::validate(*req);
    if (v != GB_OK) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->rejected++;
        return v;
    }
    const uint64_t bytes = gb::request_bytes(*req);
    if (bytes > s->cfg.hbm_budget_bytes) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->rejected++;
        return gb::set_status(GB_ERR_OOM, "gb_server_submit: request needs %llu bytes, budget is %llu",
                              (unsigned long long)bytes, (unsigned long long)s->cfg.hbm_budget_bytes);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        const double t = gb::now_s();
        if (s->submitted == 0) s->t_first = t;
        s->waiting.push_back(gb::Pending{*req, bytes, t});
        s->submitted++;
    }
    s->cv_dispatch.notify_one();
    return gb::ok();
}

int gb_server_poll(gb_server *sv, uint64_t *tags, double *latency_s, int max) {
    if (!sv || max <= 0) return 0;
    Server *s = reinterpret_cast<Server *>(sv);
    std::lock_guard<std::mutex> lk(s->mu);
    int n = (int)std::min<size_t>((size_t)max, s->done_tags.size());
    for (int i = 0; i < n; i++) {
        if (tags) tags[i] = s->done_tags[i];
        if (latency_s) latency_s[i] = s->done_lat[i];
    }
    s->done_tags.erase(s->done_tags.begin(), s->done_tags.begin() + n);
    s->done_lat.erase(s->done_lat.begin(), s->done_lat.begin() + n);
    return n;
}

gb_status gb_server_drain(gb_server *sv, double timeout_s) {
    GB_CHECK_ARG(sv != nullptr, "gb_server_drain: null server");
    Server *s = reinterpret_cast<Server *>(sv);
    std::unique_lock<std::mutex> lk(s->mu);
    auto pred = [s] { return s->completed >= s->submitted && s->waiting.empty() && s->inflight == 0; };
    if (timeout_s > 0) {
        if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
            return gb::set_status(GB_ERR_DEVICE_TIMEOUT, "gb_server_drain: %lld requests still pending after %.1f s",
                                  (long long)(s->submitted - s->completed), timeout_s);
    } else {
        s->cv_done.wait(lk, pred);
    }
    if (s->last_error != GB_OK)
        return gb::set_status((gb_status)s->last_error, "gb_server_drain: %lld request(s) failed to launch",
                              (long long)s->failed);
    return gb::ok();
}

gb_status gb_server_get_stats(gb_server *sv, gb_server_stats *out) {
    GB_CHECK_ARG(sv && out, "gb_server_get_stats: null argument");
    Server *s = reinterpret_cast<Server *>(sv);
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->rejected = s->rejected;
    out->failed = s->failed;
    out->waiting = (int64_t)s->waiting.size();
    out->inflight = s->inflight;
    out->inflight_bytes = s->inflight_bytes;
    out->launches = s->launches;
    out->grouped_launches = s->grouped_launches;
    out->grouped_requests = s->grouped_requests;
    out->graph_launches = s->graph_launches.load();
    out->graph_instantiations = s->graph_instantiations.load();
    out->urgent_launches = s->urgent_launches;
    out->p50_s = gb::percentile(s->latencies, 0.50);
    out->p99_s = gb::percentile(s->latencies, 0.99);
    out->mean_s = 0;
    for (double x : s->latencies) out->mean_s += x;
    if (!s->latencies.empty()) out->mean_s /= (double)s->latencies.size();
    const double span = s->t_last - s->t_first;
    out->req_per_s = span > 0 ? (double)s->completed / span : 0.0;
    return gb::ok();
}

void gb_server_destroy(gb_server *sv) {
    if (!sv) return;
    Server *s = reinterpret_cast<Server *>(sv);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_dispatch.notify_all();
    if (s->dispatcher.joinable()) s->dispatcher.join();
    if (!s->cfg.dry_run) {
        for (auto st : s->streams) cudaStreamSynchronize(st);
        for (auto &cache : s->execs)
            for (auto &kv : cache) cudaGraphExecDestroy(kv.second);
        gb::group_runner_destroy(s->grouped);
        for (auto st : s->streams) cudaStreamDestroy(st);
    }
    delete s;
}

// ---------------------------------------------------------------- autotune
gb_status gb_autotune_set(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K, int algo) {
    GB_CHECK_ARG(dtype_bits == 32 || dtype_bits == 64, "gb_autotune_set: dtype_bits");
    GB_CHECK_ARG(gb::is_mode(transA) && gb::is_mode(transB), "gb_autotune_set: mode");
    GB_CHECK_ARG(algo >= GB_ALGO_AUTO && algo <= GB_ALGO_FP16X3, "gb_autotune_set: algo");
    gb_tune_choice c;
    memset(&c, 0, sizeof(c));
    c.algo = algo;
    std::lock_guard<std::mutex> lk(gb::g_tune_mu);
    gb::g_tune[gb::key_of(dtype_bits, gb::is_trans(transA), gb::is_trans(transB), M, N, K)] = c;
    return gb::ok();
}

gb_status gb_autotune_lookup(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                             gb_tune_choice *out) {
    GB_CHECK_ARG(out != nullptr, "gb_autotune_lookup: null out-pointer");
    if (!gb::tuned_choice(dtype_bits, gb::is_trans(transA), gb::is_trans(transB), M, N, K, out))
        return gb::set_status(GB_ERR_INVALID_ARG, "gb_autotune_lookup: no choice for this bucket");
    return gb::ok();
}

int gb_autotune_get(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K) {
    gb_tune_choice c;
    return gb::tuned_choice(dtype_bits, gb::is_trans(transA), gb::is_trans(transB), M, N, K, &c) ? c.algo : -1;
}

namespace gb {
namespace {

// One candidate: algorithm and knobs (as in gb_gemm_opts).
gb_status run_candidate(int bits, char ta, char tb, int64_t M, int64_t N, int64_t K, const void *A, int64_t lda,
                        const void *B, int64_t ldb, void *C, const gb_tune_choice &c, void *stream) {
    gb_gemm_opts o;
    gb_gemm_opts_init(&o);
    o.stream = stream;
    o.algo = c.algo;
    o.accum_k = c.accum_k;
    o.split_k = c.split_k;
    o.ozaki_slices = c.ozaki_slices;
    return bits == 64 ? gb_dgemm(ta, tb, M, N, K, 1.0, (const double *)A, lda, (const double *)B, ldb, 0.0,
                                 (double *)C, N, &o)
                      : gb_sgemm(ta, tb, M, N, K, 1.0f, (const float *)A, lda, (const float *)B, ldb, 0.0f,
                                 (float *)C, N, &o);
}

std::vector<gb_tune_choice> candidates(int bits, int64_t M, int64_t N, int64_t K, double target_err) {
    std::vector<gb_tune_choice> v;
    auto add = [&](int algo, int accum, int split, int slices) {
        gb_tune_choice c;
        memset(&c, 0, sizeof(c));
        c.algo = algo; c.accum_k = accum; c.split_k = split; c.ozaki_slices = slices;
        v.push_back(c);
    };
    const int64_t small = M < N ? M : N;
    if (bits == 32) {
        add(GB_ALGO_SIMT, 0, 0, 0);
        if (K >= 64) add(GB_ALGO_BF16X3, 0, 0, 0);   // its split floor meets 2*K*u32 from K ~ 12: keep a margin
        add(GB_ALGO_FP16X3, 128, 0, 0);
        add(GB_ALGO_FP16X3, 256, 0, 0);
        add(GB_ALGO_BF16X6, 0, 0, 0);
    } else {
        add(GB_ALGO_ORDERED, 0, 0, 0);
        add(GB_ALGO_DMMA, 0, 0, 0);
        const int s = ozaki_pick_slices(target_err, K);
        add(GB_ALGO_OZAKI, 0, 0, s);
        if (s < 9) add(GB_ALGO_OZAKI, 0, 0, s + 1);
    }
    if (small <= 64) {
        add(GB_ALGO_SKINNY, 0, 0, 0);
        for (int sp : {1, 4, 16}) add(GB_ALGO_SKINNY, 0, sp, 0);
    }
    return v;
}

}  // namespace
}  // namespace gb

gb_status gb_autotune_gemm_ex(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K,
                              double target_err, int reps, void *stream, gb_tune_choice *best) {
    GB_CHECK_ARG(dtype_bits == 32 || dtype_bits == 64, "gb_autotune_gemm_ex: dtype_bits");
    GB_CHECK_ARG(gb::is_mode(transA) && gb::is_mode(transB), "gb_autotune_gemm_ex: mode");
    GB_CHECK_ARG(M > 0 && N > 0 && K > 0, "gb_autotune_gemm_ex: dimensions must be positive");
    GB_CHECK_ARG(target_err >= 0.0, "gb_autotune_gemm_ex: negative target_err");
    GB_CHECK_ARG(reps == 0 || (reps >= 5 && reps <= 1000), "gb_autotune_gemm_ex: reps must be 0 or 5..1000");
    if (reps == 0) reps = 5;
    const bool ta = gb::is_trans(transA), tb = gb::is_trans(transB);
    const int64_t es = dtype_bits / 8;
    const int64_t lda = ta ? M : K, ldb = tb ? K : N;
    void *A = nullptr, *B = nullptr, *C = nullptr;
    gb_status st;
    if ((st = gb_malloc(&A, (size_t)(M * K * es))) != GB_OK) return st;
    if ((st = gb_malloc(&B, (size_t)(K * N * es))) != GB_OK) { gb_free(A); return st; }
    if ((st = gb_malloc(&C, (size_t)(M * N * es))) != GB_OK) { gb_free(A); gb_free(B); return st; }
    if (dtype_bits == 64) {
        gb_fill_f64((double *)A, ta ? K : M, lda, lda, 1, 0, stream);
        gb_fill_f64((double *)B, tb ? N : K, ldb, ldb, 2, 0, stream);
    } else {
        gb_fill_f32((float *)A, ta ? K : M, lda, lda, 1, 0, stream);
        gb_fill_f32((float *)B, tb ? N : K, ldb, ldb, 2, 0, stream);
    }
    const std::vector<gb_tune_choice> cands = gb::candidates(dtype_bits, M, N, K, target_err);
    std::vector<cudaEvent_t> ev(2 * (size_t)reps);
    for (auto &e : ev) cudaEventCreate(&e);
    gb_tune_choice arg = cands[0];
    arg.ms = 1e30;
    for (const gb_tune_choice &c0 : cands) {
        gb_tune_choice c = c0;
        bool okrun = gb::run_candidate(dtype_bits, transA, transB, M, N, K, A, lda, B, ldb, C, c, stream) == GB_OK;
        double med = 0;
        for (int attempt = 0; attempt < 2 && okrun; attempt++) {
            for (int r = 0; r < reps && okrun; r++) {
                cudaEventRecord(ev[2 * r], gb::as_stream(stream));
                okrun = gb::run_candidate(dtype_bits, transA, transB, M, N, K, A, lda, B, ldb, C, c, stream) == GB_OK;
                cudaEventRecord(ev[2 * r + 1], gb::as_stream(stream));
            }
            if (!okrun || cudaStreamSynchronize(gb::as_stream(stream)) != cudaSuccess) {
                cudaGetLastError();
                okrun = false;
                break;
            }
            std::vector<float> t((size_t)reps);
            for (int r = 0; r < reps; r++) cudaEventElapsedTime(&t[r], ev[2 * r], ev[2 * r + 1]);
            std::sort(t.begin(), t.end());
            med = t[reps / 2];
            if (t[reps - 1] <= 1.3f * t[0]) break;   // steady: keep it; else measure once more
        }
        gb_clear_last_status();
        if (okrun && med < arg.ms) {
            arg = c;
            arg.ms = med;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    gb_free(A);
    gb_free(B);
    gb_free(C);
    st = gb_sync(stream);
    if (st != GB_OK) return st;
    {
        std::lock_guard<std::mutex> lk(gb::g_tune_mu);
        gb::g_tune[gb::key_of(dtype_bits, ta, tb, M, N, K)] = arg;
    }
    if (best) *best = arg;
    return gb::ok();
}

gb_status gb_autotune_gemm(int dtype_bits, char transA, char transB, int64_t M, int64_t N, int64_t K, int *best,
                           double *best_ms) {
    gb_tune_choice c;
    gb_status st = gb_autotune_gemm_ex(dtype_bits, transA, transB, M, N, K, 0.0, 5, nullptr, &c);
    if (st != GB_OK) return st;
    if (best) *best = c.algo;
    if (best_ms) *best_ms = c.ms;
    return gb::ok();
}

gb_status gb_autotune_save(const char *path) {
    GB_CHECK_ARG(path != nullptr, "gb_autotune_save: null path");
    FILE *f = fopen(path, "w");
    if (!f) return gb::set_status(GB_ERR_INVALID_ARG, "gb_autotune_save: cannot open %s", path);
    std::lock_guard<std::mutex> lk(gb::g_tune_mu);
    fprintf(f, "# bits ta tb log2M log2N log2K algo accum_k split_k slices ms\n");
    for (auto &kv : gb::g_tune)
        fprintf(f, "%d %d %d %d %d %d %d %d %d %d %.6g\n", kv.first.bits, kv.first.ta, kv.first.tb, kv.first.lm,
                kv.first.ln, kv.first.lk, kv.second.algo, kv.second.accum_k, kv.second.split_k,
                kv.second.ozaki_slices, kv.second.ms);
    fclose(f);
    return gb::ok();
}

gb_status gb_autotune_load(const char *path) {
    GB_CHECK_ARG(path != nullptr, "gb_autotune_load: null path");
    FILE *f = fopen(path, "r");
    if (!f) return gb::set_status(GB_ERR_INVALID_ARG, "gb_autotune_load: cannot open %s", path);
    char line[256];
    std::lock_guard<std::mutex> lk(gb::g_tune_mu);
    while (fgets(line, sizeof(line), f)) {
        if (line[0] == '#') continue;
        gb::TuneKey k;
        gb_tune_choice c;
        memset(&c, 0, sizeof(c));
        const int n = sscanf(line, "%d %d %d %d %d %d %d %d %d %d %lf", &k.bits, &k.ta, &k.tb, &k.lm, &k.ln, &k.lk,
                             &c.algo, &c.accum_k, &c.split_k, &c.ozaki_slices, &c.ms);
        if ((n == 7 || n >= 10) && c.algo >= GB_ALGO_AUTO && c.algo <= GB_ALGO_FP16X3 && c.split_k >= 0 &&
            c.split_k <= 64 && c.ozaki_slices >= 0 && c.ozaki_slices <= 9)
            gb::g_tune[k] = c;
    }
    fclose(f);
    return gb::ok();
}

}  // extern "C"
