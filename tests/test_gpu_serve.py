"""Grouped persistent kernel and the serving loop on the GPU.

* gb_gemm_batch: mixed FP32 / FP64, shapes, modes and semantics in one
  launch; every result against the Dot2 oracle (normwise <= 2*K*u).
* Server: a mixed request stream (small grouped GEMMs, large FP32 -> 3xBF16,
  FP64 -> Ozaki, skinny, transpose, Jacobi) gives each request the same result
  in the mix as alone -- bit-identical for transpose and Jacobi and for GEMMs
  that take the same kernel, within the normwise GEMM tolerance otherwise --
  with grouping + CUDA graphs on and with one launch per request.
* Server graphs for one-launch requests: the replays of a bucket's cached
  (and in-place updated) graph give the bits of plain launches.
"""
import numpy as np
import pytest

import oracle
from gpu_util import dev, host, op_shape, torch_cuda

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


def _gemm_case(rng, bits, M, N, K, mode, seed):
    dt = np.float64 if bits == 64 else np.float32
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, seed, dtype=dt)
    B = oracle.fill(br, bc, seed + 1, dtype=dt)
    C = oracle.fill(M, N, seed + 2, dtype=dt)
    return A, ac, B, bc, C


def _err(got, mode, M, N, K, alpha, A, lda, B, ldb, beta, C0, ldc):
    rows = np.arange(0, M, max(1, M // 50))
    cols = np.arange(0, N, max(1, N // 50))
    return oracle.normwise_error(got, mode[0], mode[1], M, N, K, alpha, A, lda, B, ldb, beta, C0, ldc, rows, cols)[0]


def test_gemm_batch_mixed(torch):
    import gbblas
    rng = np.random.default_rng(5)
    cases, descs, keep = [], [], []
    for i in range(24):
        bits = 64 if i % 3 == 0 else 32
        M, N, K = (int(x) for x in rng.integers(1, 300, size=3))
        mode = "NT"[i % 2] + "NT"[(i // 2) % 2]
        sem = i % 3
        alpha, beta = float(rng.uniform(-2, 2)), float(rng.uniform(-2, 2))
        A, lda, B, ldb, C0 = _gemm_case(rng, bits, M, N, K, mode, 100 + 10 * i)
        dA, dB, dC = dev(A), dev(B), dev(C0)
        keep += [dA, dB, dC]
        descs.append(gbblas.gemm_desc(mode[0], mode[1], M, N, K, alpha, dA, lda, dB, ldb, beta, dC, N, bits, sem))
        cases.append((bits, mode, M, N, K, alpha, A, lda, B, ldb, beta, C0, dC, sem))
    gbblas.gemm_batch(descs)
    for bits, mode, M, N, K, alpha, A, lda, B, ldb, beta, C0, dC, sem in cases:
        got = host(dC).astype(np.float64)
        if sem == gbblas.SEM_BLAS:
            e = _err(got, mode, M, N, K, alpha, A, lda, B, ldb, beta, C0, N)
        else:   # scalar beta: compare alpha*AB against the oracle after removing the scalar terms
            base = C0.astype(np.float64) if sem == gbblas.SEM_ACCUM_SCALAR_BETA else 0.0
            e = _err(got - base - beta, mode, M, N, K, alpha, A, lda, B, ldb, 0.0, None, N)
        u = 2.0 ** -53 if bits == 64 else 2.0 ** -24
        assert e <= 2 * max(K, 1) * u + 1e-300, (bits, mode, M, N, K, sem, e)


def _requests(rng):
    """(kind, bits, shape) of a mixed stream covering every route of the server."""
    reqs = []
    for i in range(12):
        n = int(rng.integers(64, 300))
        reqs.append(("gemm", 32 if i % 3 else 64, (n, n + 5, n + 9), "NT"[i % 2] + "NT"[(i // 2) % 2]))
    reqs.append(("gemm", 32, (1024, 1024, 1024), "NN"))     # 3xBF16 by AUTO
    reqs.append(("gemm", 64, (700, 600, 800), "TN"))       # Ozaki by AUTO
    reqs.append(("gemm", 32, (3000, 16, 2000), "NN"))      # skinny thinB
    reqs.append(("gemm", 32, (8, 5000, 1500), "TT"))       # skinny shortA
    reqs.append(("gemm", 64, (2500, 8, 900), "NT"))        # skinny FP64
    reqs.append(("transpose", 32, (700, 333), None))
    reqs.append(("transpose", 64, (257, 1030), None))
    reqs.append(("stencil", 32, (300, 200), 17))
    reqs.append(("stencil", 64, (129, 250), 4))
    return reqs


def _materialize(reqs):
    import gbblas
    out = []
    for j, (kind, bits, shape, extra) in enumerate(reqs):
        dt = np.float64 if bits == 64 else np.float32
        if kind == "gemm":
            M, N, K = shape
            A, lda, B, ldb, C0 = _gemm_case(None, bits, M, N, K, extra, 500 + 10 * j)
            out.append(dict(kind=kind, bits=bits, shape=shape, mode=extra, A=A, lda=lda, B=B, ldb=ldb, C0=C0,
                            alpha=0.5 + j * 0.01, beta=-1.25))
        elif kind == "transpose":
            M, N = shape
            out.append(dict(kind=kind, bits=bits, shape=shape, A=oracle.fill(M, N, 900 + j, dtype=dt)))
        else:
            M, N = shape
            G = np.ones((M + 2, N + 2), dtype=dt)
            G[1:-1, 1:-1] = oracle.fill(M, N, 950 + j, kind=1, dtype=dt)
            out.append(dict(kind=kind, bits=bits, shape=shape, iters=extra, G=G))
    return out


def _device_set(items):
    dv = []
    for it in items:
        if it["kind"] == "gemm":
            dv.append(dict(A=dev(it["A"]), B=dev(it["B"]), C=dev(it["C0"])))
        elif it["kind"] == "transpose":
            M, N = it["shape"]
            dv.append(dict(A=dev(it["A"]), B=dev(np.zeros((N, M), dtype=it["A"].dtype))))
        else:
            dv.append(dict(A=dev(it["G"]), B=dev(it["G"])))
    return dv


def _as_request(it, d, tag):
    import gbblas
    if it["kind"] == "gemm":
        M, N, K = it["shape"]
        return gbblas.request(gbblas.OP_GEMM, it["bits"], M, N, K, A=d["A"], lda=it["lda"], B=d["B"], ldb=it["ldb"],
                              C=d["C"], ldc=N, ta=it["mode"][0], tb=it["mode"][1], alpha=it["alpha"],
                              beta=it["beta"], tag=tag)
    if it["kind"] == "transpose":
        M, N = it["shape"]
        return gbblas.request(gbblas.OP_TRANSPOSE, it["bits"], M, N, A=d["A"], lda=N, B=d["B"], ldb=M, tag=tag)
    M, N = it["shape"]
    return gbblas.request(gbblas.OP_STENCIL, it["bits"], M, N, A=d["A"], C=d["B"], iters=it["iters"], tag=tag)


def _result(it, d):
    if it["kind"] == "gemm":
        return host(d["C"])
    if it["kind"] == "transpose":
        return host(d["B"])
    return host(d["B"] if it["iters"] % 2 else d["A"])


@pytest.mark.parametrize("grouped,graphs,streams", [(1, 1, 4), (0, 1, 3), (0, 0, 1)])
def test_server_results_same_alone_and_in_mix(torch, grouped, graphs, streams):
    import gbblas
    rng = np.random.default_rng(11)
    items = _materialize(_requests(rng))
    # alone: each request through its own server, drained before the next
    alone = []
    with gbblas.Server(streams=1, use_grouped=grouped, use_graphs=graphs) as s:
        for j, it in enumerate(items):
            d = _device_set([it])[0]
            s.submit(_as_request(it, d, j))
            s.drain(60.0)
            alone.append(_result(it, d))
    # in the mix: everything submitted at once
    dvs = _device_set(items)
    with gbblas.Server(streams=streams, use_grouped=grouped, use_graphs=graphs) as s:
        for j, (it, d) in enumerate(zip(items, dvs)):
            s.submit(_as_request(it, d, j))
        s.drain(120.0)
        st = s.stats()
        done = sorted(t for t, _ in s.poll())
    assert st["completed"] == len(items) and st["failed"] == 0 and done == list(range(len(items)))
    if grouped:
        assert st["grouped_requests"] >= 6 and st["grouped_launches"] >= 1
    for j, (it, d) in enumerate(zip(items, dvs)):
        mix = _result(it, d)
        if it["kind"] != "gemm":
            assert mix.tobytes() == alone[j].tobytes(), (j, it["kind"])
            continue
        M, N, K = it["shape"]
        u = 2.0 ** -53 if it["bits"] == 64 else 2.0 ** -24
        e_mix = _err(mix.astype(np.float64), it["mode"], M, N, K, it["alpha"], it["A"], it["lda"], it["B"], it["ldb"],
                     it["beta"], it["C0"], N)
        e_alone = _err(alone[j].astype(np.float64), it["mode"], M, N, K, it["alpha"], it["A"], it["lda"], it["B"],
                       it["ldb"], it["beta"], it["C0"], N)
        assert e_mix <= 2 * K * u and e_alone <= 2 * K * u, (j, it["shape"], e_mix, e_alone)
        if not grouped:   # same kernel either way: identical bits
            assert mix.tobytes() == alone[j].tobytes(), j


def _one_launch_items():
    """Requests that run one launch each (no grouping): every GEMM route with
    a workspace (3xBF16, FP16X3, BF16X6, Ozaki, skinny FP32 split-K, thin
    FP64), plain SIMT / DMMA, transpose and Jacobi."""
    import gbblas
    reqs = [("gemm", 32, (1024, 1024, 1024), "NN"), ("gemm", 32, (640, 768, 1000), "TN"),
            ("gemm", 32, (512, 512, 700), "NT"), ("gemm", 32, (300, 260, 500), "TT"),
            ("gemm", 64, (700, 600, 800), "TN"), ("gemm", 64, (200, 220, 300), "NN"),
            ("gemm", 32, (3000, 16, 20000), "NN"), ("gemm", 32, (8, 5000, 1500), "TT"),
            ("gemm", 64, (2500, 8, 900), "NT"), ("transpose", 32, (700, 333), None),
            ("transpose", 64, (257, 1030), None), ("stencil", 32, (300, 200), 17), ("stencil", 64, (129, 250), 4)]
    algos = [gbblas.ALGO_AUTO, gbblas.ALGO_FP16X3, gbblas.ALGO_BF16X6, gbblas.ALGO_SIMT, gbblas.ALGO_AUTO,
             gbblas.ALGO_DMMA, gbblas.ALGO_AUTO, gbblas.ALGO_AUTO, gbblas.ALGO_AUTO] + [gbblas.ALGO_AUTO] * 4
    return _materialize(reqs), algos


def test_server_one_launch_requests_replay_graphs_bit_identical(torch):
    """Three requests of one bucket in a row, each on fresh buffers: the first
    runs as plain launches, the second is captured and instantiated, the third
    updates the cached graph in place.  All three give the bits one plain
    launch gives, and the second and third are graph replays."""
    import gbblas
    items, algos = _one_launch_items()
    for j, (it, algo) in enumerate(zip(items, algos)):
        d = _device_set([it])[0]
        with gbblas.Server(streams=1, use_grouped=0, use_graphs=0) as s:
            r = _as_request(it, d, 0)
            r.algo = algo
            s.submit(r)
            s.drain(60.0)
            assert s.stats()["failed"] == 0
        want = _result(it, d)
        with gbblas.Server(streams=1, use_grouped=0, use_graphs=1) as s:
            for rep in range(3):
                d = _device_set([it])[0]
                r = _as_request(it, d, rep)
                r.algo = algo
                s.submit(r)
                s.drain(60.0)
                assert _result(it, d).tobytes() == want.tobytes(), (j, it["kind"], it.get("shape"), rep)
            st = s.stats()
        assert st["failed"] == 0 and st["completed"] == 3
        assert st["graph_launches"] == 2 and st["graph_instantiations"] == 1, (j, it["kind"], it.get("shape"), st)


def test_autotune_picks_a_working_algorithm(torch):
    import gbblas
    best, ms = gbblas.autotune_gemm(32, "N", "N", 1024, 1024, 1024)
    assert best in (gbblas.ALGO_SIMT, gbblas.ALGO_BF16X3, gbblas.ALGO_FP16X3, gbblas.ALGO_BF16X6) and ms > 0
    assert gbblas.lib().gb_autotune_get(32, b"N", b"N", 1024, 1024, 1024) == best
    best64, _ = gbblas.autotune_gemm(64, "N", "N", 600, 600, 600)
    assert best64 in (gbblas.ALGO_ORDERED, gbblas.ALGO_OZAKI, gbblas.ALGO_DMMA)


@pytest.mark.parametrize("bits,mode,M,N,K,target", [(32, "NT", 2048, 1536, 1024, 0.0), (64, "NN", 1024, 768, 2048, 1e-12),
                                                     (64, "TN", 1024, 1024, 1024, 0.0), (32, "TN", 16, 30000, 4096, 0.0),
                                                     (64, "NN", 40000, 24, 2048, 0.0)])
def test_autotune_ex_choice_runs_within_its_bound(torch, bits, mode, M, N, K, target):
    """The tuner's choice (algorithm and knobs) is stored for the bucket, was
    timed on the stream given, and computes the product within 2*K*u (or the
    Ozaki target) when run through the server on fresh inputs."""
    import gbblas
    tc = torch
    s = tc.cuda.Stream()
    ta, tb = mode
    c = gbblas.autotune_gemm_ex(bits, ta, tb, M, N, K, target_err=target, reps=5, stream=s)
    assert c["ms"] > 0
    assert gbblas.autotune_lookup(bits, ta, tb, M, N, K) == c
    dtype = np.float64 if bits == 64 else np.float32
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, 201, dtype=dtype)
    B = oracle.fill(br, bc, 202, dtype=dtype)
    C0 = oracle.fill(M, N, 203, dtype=dtype)
    dA, dB, dC = dev(A), dev(B), dev(C0)
    with gbblas.Server(streams=2) as srv:
        srv.submit(gbblas.request(gbblas.OP_GEMM, bits, M, N, K, dA, ac, dB, bc, dC, N, ta=ta, tb=tb, alpha=0.5,
                                  beta=-1.0, tag=1))
        srv.drain(60.0)
    rows = np.arange(0, M, max(1, M // 64))
    cols = np.arange(0, N, max(1, N // 64))
    err, _ = oracle.normwise_error(host(dC), ta, tb, M, N, K, 0.5, A, ac, B, bc, -1.0, C0, N, rows, cols)
    u = 2.0 ** -53 if bits == 64 else 2.0 ** -24
    bound = target if (bits == 64 and target > 0 and c["algo"] == gbblas.ALGO_OZAKI) else 2 * K * u
    assert err <= bound, (c, err)


@pytest.mark.parametrize("split", [1, 3, 16])
@pytest.mark.parametrize("bits", [32, 64])
def test_skinny_split_k_override(torch, split, bits):
    """split_k overrides the planner's split-K: every count gives the product
    within 2*K*u (thinB and shortA)."""
    import gbblas
    dtype = np.float64 if bits == 64 else np.float32
    u = 2.0 ** -53 if bits == 64 else 2.0 ** -24
    for M, N, mode in ((6000, 12, "NN"), (24, 5000, "TT")):
        K = 9000
        ta, tb = mode
        ar, ac = op_shape(ta, M, K)
        br, bc = op_shape(tb, K, N)
        A = oracle.fill(ar, ac, 211, dtype=dtype)
        B = oracle.fill(br, bc, 212, dtype=dtype)
        C0 = oracle.fill(M, N, 213, dtype=dtype)
        dC = dev(C0)
        gbblas.gemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, 0.5, dC, N, bits, algo=gbblas.ALGO_SKINNY,
                    split_k=split)
        rows = np.arange(0, M, max(1, M // 50))
        cols = np.arange(0, N, max(1, N // 50))
        err, _ = oracle.normwise_error(host(dC), ta, tb, M, N, K, 1.0, A, ac, B, bc, 0.5, C0, N, rows, cols)
        assert err <= 2 * K * u, (mode, split, err)


@pytest.mark.parametrize("algo_name,accum", [("FP16X3", 32), ("FP16X3", 512), ("FP16X3", -1), ("BF16X3", 256),
                                             ("BF16X6", -1), ("BF16X6", 128)])
def test_accum_k_knob(torch, algo_name, accum):
    """accum_k sets the accumulator chunk of the tensor-core SGEMM forms: exact
    on small integers, within 2*K*u32 on U[-1,1]."""
    import gbblas
    algo = getattr(gbblas, "ALGO_" + algo_name)
    M, N, K = 640, 520, 1500
    rng = np.random.default_rng(214)
    A = rng.integers(-8, 9, size=(M, K)).astype(np.float32)
    B = rng.integers(-8, 9, size=(K, N)).astype(np.float32)
    dC = dev(np.zeros((M, N), np.float32))
    gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=algo, accum_k=accum)
    assert np.array_equal(host(dC), (A.astype(np.float64) @ B.astype(np.float64)).astype(np.float32))
    A = oracle.fill(M, K, 215, dtype=np.float32)
    B = oracle.fill(K, N, 216, dtype=np.float32)
    dC = dev(np.zeros((M, N), np.float32))
    gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=algo, accum_k=accum)
    err, _ = oracle.normwise_error(host(dC), "N", "N", M, N, K, 1.0, A, K, B, N, 0.0, None, N,
                                   np.arange(0, M, 5), np.arange(0, N, 5))
    assert err <= 2 * K * 2.0 ** -24 + (3 * 2.0 ** -17 if algo_name == "BF16X3" else 0), err


def test_strided_batched_matches_single_calls(torch):
    """gb_gemm_strided_batched: 37 equal-shape GEMMs through the grouped kernel
    equal 37 single gb_dgemm calls with the ordered algorithm on FP64 within
    the normwise bound, and shared operands (stride 0) work."""
    import gbblas
    batch, M, N, K = 37, 70, 90, 130
    A = oracle.fill(batch * M, K, 71, dtype=np.float64)
    B = oracle.fill(K, N, 72, dtype=np.float64)            # shared: strideB = 0
    C0 = oracle.fill(batch * M, N, 73, dtype=np.float64)
    dC = dev(C0)
    gbblas.gemm_strided_batched(64, "N", "N", M, N, K, 1.25, dev(A), K, M * K, dev(B), N, 0, -0.5, dC, N, M * N,
                                batch)
    got = host(dC)
    for i in range(batch):
        Ai, Ci = A[i * M:(i + 1) * M], C0[i * M:(i + 1) * M]
        err, _ = oracle.normwise_error(got[i * M:(i + 1) * M], "N", "N", M, N, K, 1.25, Ai, K, B, N, -0.5, Ci, N)
        assert err <= 2 * K * 2.0 ** -53, (i, err)
