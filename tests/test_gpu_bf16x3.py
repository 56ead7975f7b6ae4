"""3xBF16 SGEMM on tcgen05 against the oracle.

* Small-integer inputs: the hi/lo split is exact and every partial sum is an
  integer below 2^24, so the result must equal the exact product bit for
  bit -- this pins the TMA / UMMA descriptor layouts and the TMEM epilogue.
* U[-1,1] inputs: normwise error against the Dot2 oracle <= 2*K*u32 plus
  the split's own representation error: hi + lo keeps ~16 of FP32's 24
  bits, so each product carries up to ~3 * 2^-17 relative error however
  small K is (below K ~ 12 that exceeds 2*K*u32 alone).
"""

SPLIT_ERR = 3 * 2.0 ** -17
# FP16X3 error at K = 4096 relative to plain FFMA on the same inputs (at most)
FP16X3_VS_SIMT = 1.0
import numpy as np
import pytest

import oracle
from gpu_util import dev, host, op_shape, torch_cuda

pytestmark = pytest.mark.gpu
MODES = ["NN", "NT", "TN", "TT"]


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


def _ints(rows, cols, seed, ld=None):
    rng = np.random.default_rng(seed)
    X = np.zeros((rows, ld or cols), dtype=np.float32)
    X[:, :cols] = rng.integers(-8, 9, size=(rows, cols)).astype(np.float32)
    return X


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (256, 512, 192), (130, 300, 70), (7, 9, 5), (1030, 2050, 96),
                                   (2048, 4096, 64)])
def test_bf16x3_exact_on_integers(torch, mode, M, N, K):
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A, B = _ints(ar, ac, 1), _ints(br, bc, 2)
    C0 = _ints(M, N, 3)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    want = (2.0 * (opA.astype(np.float64) @ opB.astype(np.float64)) + 1.0 * C0).astype(np.float32)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 2.0, dev(A), ac, dev(B), bc, 1.0, dC, N, algo=gbblas.ALGO_BF16X3)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, bad[:5], got[tuple(bad[0])] if bad.size else None)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K,pad", [(384, 512, 1040, 16), (333, 257, 515, 3), (1, 1, 1, 0), (129, 1000, 4096, 8)])
def test_bf16x3_normwise(torch, mode, M, N, K, pad):
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, 31, dtype=np.float32, ld=ac + pad)
    B = oracle.fill(br, bc, 32, dtype=np.float32, ld=bc + pad)
    C0 = oracle.fill(M, N, 33, dtype=np.float32, ld=N + pad)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 1.5, dev(A), ac + pad, dev(B), bc + pad, -0.5, dC, N + pad,
                 algo=gbblas.ALGO_BF16X3)
    got = host(dC)
    rows = np.arange(0, M, max(1, M // 97))
    cols = np.arange(0, N, max(1, N // 97))
    err, _ = oracle.normwise_error(got, ta, tb, M, N, K, 1.5, A, ac + pad, B, bc + pad, -0.5, C0, N + pad,
                                   rows, cols)
    assert err <= 2 * K * 2.0 ** -24 + SPLIT_ERR, err
    if K >= 64:
        assert err <= 2 * K * 2.0 ** -24, err
    # columns beyond N (the ld padding) are untouched
    if pad:
        assert np.array_equal(got[:, N:], C0[:, N:])


@pytest.mark.parametrize("sem", [1, 2])
def test_bf16x3_scalar_beta_semantics(torch, sem):
    import gbblas
    M, N, K = 200, 300, 128
    A = _ints(M, K, 4)
    B = _ints(K, N, 5)
    C0 = _ints(M, N, 6)
    exact = (1.5 * (A.astype(np.float64) @ B.astype(np.float64)))
    want = (exact + 3.0) if sem == 1 else (C0 + (exact + 3.0))
    dC = dev(C0)
    gbblas.sgemm("N", "N", M, N, K, 1.5, dev(A), K, dev(B), N, 3.0, dC, N, algo=gbblas.ALGO_BF16X3, semantics=sem)
    assert np.array_equal(host(dC), want.astype(np.float32))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K", [(300, 16, 128), (257, 40, 96), (1000, 100, 64), (129, 300, 160), (640, 8, 4096)])
def test_bf16x3_fused_tile_widths_exact(torch, mode, M, N, K):
    """Aligned leading dimensions can take the fused-split kernel (forced
    here); N picks the 32/64/128/256-wide tile.  Small integers: exact."""
    import os
    import gbblas
    os.environ["GB_BF16X3_PATH"] = "fused"
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    pa, pb = (-ac) % 4, (-bc) % 4            # pad leading dimensions to a multiple of 4
    A, B, C0 = _ints(ar, ac, 7, ld=ac + pa), _ints(br, bc, 8, ld=bc + pb), _ints(M, N, 9)
    opA = A[:, :ac].T if ta == "T" else A[:, :ac]
    opB = B[:, :bc].T if tb == "T" else B[:, :bc]
    want = (-1.0 * (opA.astype(np.float64) @ opB.astype(np.float64)) + 0.5 * C0).astype(np.float32)
    dC = dev(C0)
    try:
        gbblas.sgemm(ta, tb, M, N, K, -1.0, dev(A), ac + pa, dev(B), bc + pb, 0.5, dC, N, algo=gbblas.ALGO_BF16X3)
    finally:
        os.environ.pop("GB_BF16X3_PATH", None)
    got = host(dC)
    assert np.array_equal(got, want), (mode, np.argwhere(got != want)[:4])


def test_bf16x3_fused_matches_two_pass(torch):
    import os
    import gbblas
    M, N, K = 700, 520, 2000
    A = oracle.fill(M, K, 51, dtype=np.float32)
    B = oracle.fill(N, K, 52, dtype=np.float32)
    C0 = oracle.fill(M, N, 53, dtype=np.float32)
    outs = []
    for path in ("fused", "two-pass"):
        os.environ["GB_BF16X3_PATH"] = path
        try:
            dC = dev(C0)
            gbblas.sgemm("N", "T", M, N, K, 1.25, dev(A), K, dev(B), K, -0.75, dC, N, algo=gbblas.ALGO_BF16X3)
            outs.append(host(dC))
        finally:
            os.environ.pop("GB_BF16X3_PATH", None)
    # same products, same per-K-step MMA order: identical results
    assert outs[0].tobytes() == outs[1].tobytes()


# ---------------------------------------------------------------- BF16X6
# Three BF16 pieces per operand (hi, mid, lo: 24 significand bits, so any
# FP32 value of normal range is carried exactly) and the six piece products
# of combined weight >= 2^-16.  The dropped products (mid*lo, lo*mid, lo*lo)
# and the representation residue sum to about 2^-25 relative, below u32, so
# the error is the FP32 accumulation's own.

@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (130, 300, 70), (7, 9, 5), (1030, 700, 96)])
def test_bf16x6_exact_on_integers(torch, mode, M, N, K):
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A, B = _ints(ar, ac, 11), _ints(br, bc, 12)
    C0 = _ints(M, N, 13)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    want = (2.0 * (opA.astype(np.float64) @ opB.astype(np.float64)) - 1.0 * C0).astype(np.float32)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 2.0, dev(A), ac, dev(B), bc, -1.0, dC, N, algo=gbblas.ALGO_BF16X6)
    got = host(dC)
    assert np.array_equal(got, want), (mode, np.argwhere(got != want)[:5])


@pytest.mark.parametrize("mode", MODES)
def test_bf16x6_carries_24_bits(torch, mode):
    """A holds 20-bit integers (hi + lo alone carry 16 bits): only the
    three-piece split reproduces the products exactly."""
    import gbblas
    ta, tb = mode
    M, N, K = 256, 384, 8
    rng = np.random.default_rng(14)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = rng.integers(-(1 << 19), 1 << 19, size=(ar, ac)).astype(np.float32)
    B = rng.integers(-3, 4, size=(br, bc)).astype(np.float32)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    want = (opA.astype(np.float64) @ opB.astype(np.float64)).astype(np.float32)   # |sum| < 2^24: exact
    dC = dev(np.zeros((M, N), np.float32))
    gbblas.sgemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, 0.0, dC, N, algo=gbblas.ALGO_BF16X6)
    got = host(dC)
    assert np.array_equal(got, want), (mode, np.argwhere(got != want)[:5])
    dC3 = dev(np.zeros((M, N), np.float32))
    gbblas.sgemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, 0.0, dC3, N, algo=gbblas.ALGO_BF16X3)
    assert not np.array_equal(host(dC3), want)   # two pieces lose the low bits


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K,pad", [(384, 512, 1040, 16), (333, 257, 515, 3), (1, 1, 1, 0), (129, 1000, 4096, 8),
                                       (64, 64, 3, 1)])
def test_bf16x6_normwise_fp32_level(torch, mode, M, N, K, pad):
    """Unlike BF16X3 there is no split floor: the FP32 bound holds at any K."""
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, 41, dtype=np.float32, ld=ac + pad)
    B = oracle.fill(br, bc, 42, dtype=np.float32, ld=bc + pad)
    C0 = oracle.fill(M, N, 43, dtype=np.float32, ld=N + pad)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 1.5, dev(A), ac + pad, dev(B), bc + pad, -0.5, dC, N + pad,
                 algo=gbblas.ALGO_BF16X6)
    got = host(dC)
    rows = np.arange(0, M, max(1, M // 97))
    cols = np.arange(0, N, max(1, N // 97))
    err, _ = oracle.normwise_error(got, ta, tb, M, N, K, 1.5, A, ac + pad, B, bc + pad, -0.5, C0, N + pad,
                                   rows, cols)
    assert err <= (2 * K + 4) * 2.0 ** -24, err
    if pad:
        assert np.array_equal(got[:, N:], C0[:, N:])


def test_bf16x6_error_tracks_simt(torch):
    """At K = 4096 the six-product result is as accurate as plain FFMA
    (within 2x), and an order of magnitude better than three products."""
    import gbblas
    M = N = 512
    K = 4096
    A = oracle.fill(M, K, 61, dtype=np.float32)
    B = oracle.fill(K, N, 62, dtype=np.float32)
    C0 = np.zeros((M, N), np.float32)
    rows = np.arange(0, M, 8)
    cols = np.arange(0, N, 8)
    errs = {}
    for name, algo in (("simt", gbblas.ALGO_SIMT), ("x3", gbblas.ALGO_BF16X3), ("x6", gbblas.ALGO_BF16X6)):
        dC = dev(C0)
        gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=algo)
        errs[name], _ = oracle.normwise_error(host(dC), "N", "N", M, N, K, 1.0, A, K, B, N, 0.0, C0, N, rows, cols)
    assert errs["x6"] <= 2 * errs["simt"], errs
    assert errs["x6"] * 4 <= errs["x3"], errs


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K", [(4096, 4096, 96), (1152, 4352, 64), (300, 700, 128)])
def test_bf16x3_half_tile_tail_exact(torch, mode, M, N, K):
    """A last wave at most half full runs as 128-column half tiles (N = 128
    MMAs on the first half of the B stage); small integers: exact."""
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A, B = _ints(ar, ac, 41), _ints(br, bc, 42)
    C0 = _ints(M, N, 43)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    want = (3.0 * (opA.astype(np.float64) @ opB.astype(np.float64)) + 1.0 * C0).astype(np.float32)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 3.0, dev(A), ac, dev(B), bc, 1.0, dC, N, algo=gbblas.ALGO_BF16X3)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, bad[:5])


@pytest.mark.parametrize("algo_name", ["BF16X3", "BF16X6"])
def test_back_to_back_calls_overlap_safely(torch, algo_name):
    """Calls issued back to back on one stream: each call's split pass may run
    beside the previous call's GEMM (programmatic dependent launch, pieces in
    alternating workspace halves).  A chain C <- A_i B_i + C over eight
    calls with different operands must give the same bits as the calls run
    one after another (GB_BF16X3_PDL=0)."""
    import os
    import gbblas
    algo = getattr(gbblas, "ALGO_" + algo_name)
    M, N, K = 1536, 1280, 1024
    As = [dev(oracle.fill(M, K, 300 + i, dtype=np.float32)) for i in range(8)]
    Bs = [dev(oracle.fill(K, N, 400 + i, dtype=np.float32)) for i in range(8)]
    C0 = oracle.fill(M, N, 500, dtype=np.float32)
    outs = []
    for pdl in ("1", "0"):
        os.environ["GB_BF16X3_PDL"] = pdl
        try:
            dC = dev(C0)
            for i in range(8):   # no host synchronisation between the calls
                mode = "NN" if i % 2 == 0 else "NT"
                B = Bs[i] if mode == "NN" else Bs[i].t().contiguous()
                ldb = N if mode == "NN" else K
                gbblas.sgemm(mode[0], mode[1], M, N, K, 1.0, As[i], K, B, ldb, 1.0, dC, N, algo=algo)
            outs.append(host(dC))
        finally:
            os.environ.pop("GB_BF16X3_PDL", None)
    assert outs[0].tobytes() == outs[1].tobytes()


def test_back_to_back_calls_of_mixed_sizes(torch):
    """Large and small calls alternating without host synchronisation: a small
    call's split pass (beside the large call's GEMM) writes its own half of
    the workspace wherever the large call's pieces end.  Same bits as the
    calls run one after another."""
    import os
    import gbblas
    shapes = [(2048, 1792, 2048), (384, 256, 320), (1536, 2048, 1024), (256, 512, 768)]
    ops = [(dev(oracle.fill(M, K, 600 + i, dtype=np.float32)), dev(oracle.fill(K, N, 700 + i, dtype=np.float32)))
           for i, (M, N, K) in enumerate(shapes)]
    outs = []
    for pdl in ("1", "0"):
        os.environ["GB_BF16X3_PDL"] = pdl
        try:
            Cs = [dev(oracle.fill(M, N, 800 + i, dtype=np.float32)) for i, (M, N, K) in enumerate(shapes)]
            for rep in range(3):
                for i, (M, N, K) in enumerate(shapes):
                    A, B = ops[i]
                    gbblas.sgemm("N", "N", M, N, K, 1.0, A, K, B, N, 1.0, Cs[i], N, algo=gbblas.ALGO_BF16X3)
            outs.append([host(c).tobytes() for c in Cs])
        finally:
            os.environ.pop("GB_BF16X3_PDL", None)
    assert outs[0] == outs[1]


def _pdl_both(fn):
    """fn() run with the split passes allowed beside the previous GEMM and
    with every launch in plain stream order (GB_BF16X3_PDL=0)."""
    import os
    outs = []
    for pdl in ("1", "0"):
        os.environ["GB_BF16X3_PDL"] = pdl
        try:
            outs.append(fn())
        finally:
            os.environ.pop("GB_BF16X3_PDL", None)
    return outs


@pytest.mark.parametrize("algo_name", ["bf16x3", "fp16x3"])
def test_back_to_back_chain_reads_previous_result(torch, algo_name):
    """C1 = A B, then C2 = C1 D, then C3 = E C2 with no host synchronisation:
    each call's operands are the previous call's result, so no scan or split
    may read them before the GEMM that writes them has finished.  Same bits
    as the calls in plain order."""
    import gbblas
    algo = gbblas.ALGO_BF16X3 if algo_name == "bf16x3" else gbblas.ALGO_FP16X3
    M = N = K = 1536
    A = dev(oracle.fill(M, K, 901, dtype=np.float32))
    D = dev(oracle.fill(K, N, 902, dtype=np.float32))
    E = dev(oracle.fill(M, K, 903, dtype=np.float32))

    def run():
        C1 = dev(np.zeros((M, N), np.float32))
        C2 = dev(np.zeros((M, N), np.float32))
        C3 = dev(np.zeros((M, N), np.float32))
        gbblas.sgemm("N", "N", M, N, K, 1.0, A, K, D, N, 0.0, C1, N, algo=algo)
        gbblas.sgemm("N", "N", M, N, K, 0.5, C1, N, D, N, 0.0, C2, N, algo=algo)
        gbblas.sgemm("N", "T", M, N, K, 0.25, E, K, C2, N, 0.0, C3, N, algo=algo)
        return host(C3).tobytes()

    a, b = _pdl_both(run)
    assert a == b


def test_back_to_back_alternating_forms(torch):
    """BF16X3, BF16X6 and FP16X3 calls alternating on one stream with no host
    synchronisation: every two-pass call places its pieces in the same two
    workspace halves, whatever the form of the previous call.  Same bits as
    the calls in plain order."""
    import gbblas
    shapes = [(1536, 1280, 1024), (640, 768, 512), (2048, 1024, 768)]
    ops = [(dev(oracle.fill(M, K, 920 + i, dtype=np.float32)), dev(oracle.fill(K, N, 930 + i, dtype=np.float32)))
           for i, (M, N, K) in enumerate(shapes)]
    algos = [gbblas.ALGO_BF16X3, gbblas.ALGO_BF16X6, gbblas.ALGO_FP16X3]

    def run():
        Cs = [dev(oracle.fill(M, N, 940 + i, dtype=np.float32)) for i, (M, N, K) in enumerate(shapes)]
        for rep in range(3):
            for i, (M, N, K) in enumerate(shapes):
                A, B = ops[i]
                gbblas.sgemm("N", "N", M, N, K, 1.0, A, K, B, N, 1.0, Cs[i], N, algo=algos[(i + rep) % 3])
        return [host(c).tobytes() for c in Cs]

    a, b = _pdl_both(run)
    assert a == b


@pytest.mark.parametrize("algo_name", ["bf16x3", "fp16x3"])
def test_back_to_back_with_caller_work_in_between(torch, algo_name):
    """A torch kernel on the same stream rewrites the next call's B between
    two calls: the next call's scan and split start only after that kernel
    and read the new B.  Same bits as the calls in plain order."""
    import gbblas
    algo = gbblas.ALGO_BF16X3 if algo_name == "bf16x3" else gbblas.ALGO_FP16X3
    tc = torch
    M = N = K = 1024
    A = dev(oracle.fill(M, K, 950, dtype=np.float32))
    B0 = dev(oracle.fill(K, N, 951, dtype=np.float32))
    B1src = dev(oracle.fill(K, N, 952, dtype=np.float32))

    def run():
        B1 = tc.zeros_like(B1src)
        C0 = dev(np.zeros((M, N), np.float32))
        C1 = dev(np.zeros((M, N), np.float32))
        tc.cuda.synchronize()
        gbblas.sgemm("N", "N", M, N, K, 1.0, A, K, B0, N, 0.0, C0, N, algo=algo)
        B1.copy_(B1src)          # torch's current stream is the legacy default stream gbblas uses
        gbblas.sgemm("N", "N", M, N, K, 1.0, A, K, B1, N, 0.0, C1, N, algo=algo)
        return host(C0).tobytes() + host(C1).tobytes()

    a, b = _pdl_both(run)
    assert a == b


def test_fp16x3_back_to_back_overlapped_scans(torch):
    """FP16X3 calls in a row with disjoint operands (scan and split of each
    call beside the previous call's GEMM), every layout and a ragged shape,
    the line maxima kept between calls (generation tags, no clearing): same
    bits as the calls in plain order, and as each call alone."""
    import gbblas
    shapes = [(1536, 1280, 1024, "NN"), (640, 768, 512, "TN"), (1000, 1100, 700, "NT"), (2048, 1024, 768, "TT")]
    ops = []
    for i, (M, N, K, mode) in enumerate(shapes):
        ar, ac = op_shape(mode[0], M, K)
        br, bc = op_shape(mode[1], K, N)
        ops.append((dev(oracle.fill(ar, ac, 960 + i, dtype=np.float32)), ac,
                    dev(oracle.fill(br, bc, 970 + i, dtype=np.float32)), bc))

    def run():
        Cs = [dev(oracle.fill(M, N, 980 + i, dtype=np.float32)) for i, (M, N, K, mode) in enumerate(shapes)]
        for rep in range(3):
            for i, (M, N, K, mode) in enumerate(shapes):
                A, lda, B, ldb = ops[i]
                gbblas.sgemm(mode[0], mode[1], M, N, K, 0.75, A, lda, B, ldb, 0.5, Cs[i], N, algo=gbblas.ALGO_FP16X3)
        return [host(c).tobytes() for c in Cs]

    a, b = _pdl_both(run)
    assert a == b
    # one call alone (synchronised before and after) equals the first round of the chain
    i = 2
    M, N, K, mode = shapes[i]
    A, lda, B, ldb = ops[i]
    C = dev(oracle.fill(M, N, 980 + i, dtype=np.float32))
    torch.cuda.synchronize()
    gbblas.sgemm(mode[0], mode[1], M, N, K, 0.75, A, lda, B, ldb, 0.5, C, N, algo=gbblas.ALGO_FP16X3)
    torch.cuda.synchronize()
    C1 = dev(oracle.fill(M, N, 980 + i, dtype=np.float32))
    for _ in range(2):   # other calls in between leave other generations in the maxima
        gbblas.sgemm("N", "N", 640, 768, 512, 1.0, ops[1][0], 512, ops[1][2], 768, 0.0,
                     dev(np.zeros((640, 768), np.float32)), 768, algo=gbblas.ALGO_FP16X3)
    gbblas.sgemm(mode[0], mode[1], M, N, K, 0.75, A, lda, B, ldb, 0.5, C1, N, algo=gbblas.ALGO_FP16X3)
    assert host(C).tobytes() == host(C1).tobytes()


@pytest.mark.parametrize("algo_name,accum", [("bf16x3", 0), ("fp16x3", 0), ("bf16x3", 128), ("fp16x3", 256)])
def test_half_tile_tail_bit_identical(torch, algo_name, accum):
    """A last wave at most half full runs as half tiles (128 columns) on twice
    as many CTAs (by default for the one-accumulator form; the folding form
    when GB_BF16X3_HALF=1): the same bits as whole tiles (GB_BF16X3_HALF=0).
    Shapes with 8 / 12 tail tiles for 152 / 148 SMs, and a ragged one."""
    import os
    import gbblas
    algo = gbblas.ALGO_BF16X3 if algo_name == "bf16x3" else gbblas.ALGO_FP16X3
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for M, N, K in ((128 * 10, 256 * 16, 512), (128 * ((sms + 6) // 16) + 50, 256 * 16 + 100, 300)):
        A = dev(oracle.fill(M, K, 991, dtype=np.float32))
        B = dev(oracle.fill(K, N, 992, dtype=np.float32))
        C0 = oracle.fill(M, N, 993, dtype=np.float32)
        outs = []
        for half in ("1", "0"):
            os.environ["GB_BF16X3_HALF"] = half
            try:
                C = dev(C0)
                gbblas.sgemm("N", "N", M, N, K, 1.5, A, K, B, N, -0.5, C, N, algo=algo, accum_k=accum)
                outs.append(host(C).tobytes())
            finally:
                os.environ.pop("GB_BF16X3_HALF", None)
        assert outs[0] == outs[1], (M, N, K)


# ---------------------------------------------------------------- FP16X3
# Two FP16 pieces (11 + 11 significand bits) of every value after its row of
# op(A) / column of op(B) is scaled by a power of two that puts the line's
# largest magnitude in [2^14, 2^15); the three products hi*hi + hi*lo + lo*hi,
# accumulated in chunks of 128 k that are summed in registers.  The dropped
# lo*lo term and the residue are ~2^-22 of a product, so the error is that of
# FP32 accumulation.

@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (130, 300, 70), (7, 9, 5), (1030, 2050, 96), (2048, 4096, 64)])
def test_fp16x3_exact_on_integers(torch, mode, M, N, K):
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A, B = _ints(ar, ac, 21), _ints(br, bc, 22)
    C0 = _ints(M, N, 23)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    want = (2.0 * (opA.astype(np.float64) @ opB.astype(np.float64)) + 1.0 * C0).astype(np.float32)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 2.0, dev(A), ac, dev(B), bc, 1.0, dC, N, algo=gbblas.ALGO_FP16X3)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, bad[:5])


@pytest.mark.parametrize("mode", MODES)
def test_fp16x3_exact_across_exponent_range(torch, mode):
    """Rows of op(A) and columns of op(B) scaled by powers of two from 2^-146
    (FP32 subnormals) to 2^60: each line gets its own scale, so small-integer
    products stay exact and land at the right exponent."""
    import gbblas
    ta, tb = mode
    M, N, K = 160, 144, 96
    rng = np.random.default_rng(24)
    ea = rng.choice([-146, -100, -60, -20, 0, 30, 60], size=M)
    fb = rng.choice([-60, -20, 0, 10, 50], size=N)
    opA = (rng.integers(-8, 9, size=(M, K)) * np.exp2(ea)[:, None]).astype(np.float64)
    opB = (rng.integers(-8, 9, size=(K, N)) * np.exp2(fb)[None, :]).astype(np.float64)
    want = (opA @ opB).astype(np.float32)          # every sum exact (|int sum| < 2^13)
    assert np.array_equal(opA.astype(np.float32).astype(np.float64), opA)
    A = np.ascontiguousarray(opA.T if ta == "T" else opA).astype(np.float32)
    B = np.ascontiguousarray(opB.T if tb == "T" else opB).astype(np.float32)
    dC = dev(np.zeros((M, N), np.float32))
    gbblas.sgemm(ta, tb, M, N, K, 1.0, dev(A), A.shape[1], dev(B), B.shape[1], 0.0, dC, N,
                 algo=gbblas.ALGO_FP16X3)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, bad[:5], got[tuple(bad[0])] if bad.size else None)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K,pad", [(384, 512, 1040, 16), (333, 257, 515, 3), (1, 1, 1, 0), (129, 1000, 4096, 8),
                                       (64, 64, 3, 1)])
def test_fp16x3_normwise_fp32_level(torch, mode, M, N, K, pad):
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, 71, dtype=np.float32, ld=ac + pad)
    B = oracle.fill(br, bc, 72, dtype=np.float32, ld=bc + pad)
    C0 = oracle.fill(M, N, 73, dtype=np.float32, ld=N + pad)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 1.5, dev(A), ac + pad, dev(B), bc + pad, -0.5, dC, N + pad,
                 algo=gbblas.ALGO_FP16X3)
    got = host(dC)
    rows = np.arange(0, M, max(1, M // 97))
    cols = np.arange(0, N, max(1, N // 97))
    err, _ = oracle.normwise_error(got, ta, tb, M, N, K, 1.5, A, ac + pad, B, bc + pad, -0.5, C0, N + pad,
                                   rows, cols)
    assert err <= (2 * K + 4) * 2.0 ** -24, err
    if pad:
        assert np.array_equal(got[:, N:], C0[:, N:])


def test_fp16x3_error_tracks_simt(torch):
    """At K = 4096 the FP16 three-product result is as accurate as plain
    FFMA, and an order of magnitude better than BF16X3."""
    import gbblas
    M = N = 512
    K = 4096
    A = oracle.fill(M, K, 81, dtype=np.float32)
    B = oracle.fill(K, N, 82, dtype=np.float32)
    C0 = np.zeros((M, N), np.float32)
    rows = np.arange(0, M, 8)
    cols = np.arange(0, N, 8)
    errs = {}
    for name, algo in (("simt", gbblas.ALGO_SIMT), ("x3", gbblas.ALGO_BF16X3), ("f16", gbblas.ALGO_FP16X3)):
        dC = dev(C0)
        gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=algo)
        errs[name], _ = oracle.normwise_error(host(dC), "N", "N", M, N, K, 1.0, A, K, B, N, 0.0, C0, N, rows, cols)
    assert errs["f16"] <= errs["simt"] * FP16X3_VS_SIMT, errs
    assert errs["f16"] * 4 <= errs["x3"], errs


@pytest.mark.parametrize("mode", ["NN", "TT"])
def test_fp16x3_inf_nan_propagate(torch, mode):
    """A row of op(A) holding +Inf, one holding NaN and a column of op(B)
    holding -Inf: those outputs are plain FP32 dot products, so NaN and
    +-Inf appear exactly where IEEE arithmetic puts them; the rest is
    unaffected."""
    import gbblas
    ta, tb = mode
    M, N, K = 300, 280, 200
    opA = oracle.fill(M, K, 91, dtype=np.float32)
    opB = oracle.fill(K, N, 92, dtype=np.float32)
    opA[3, 17] = np.inf
    opA[7, 40] = np.nan
    opB[55, 5] = -np.inf
    opB[:, 9] = 0.0
    opB[60, 9] = np.inf      # column 9: Inf times the zeros of op(A)'s row 11
    opA[11, :] = 0.0
    opA[11, 60] = 1.0
    A = np.ascontiguousarray(opA.T if ta == "T" else opA)
    B = np.ascontiguousarray(opB.T if tb == "T" else opB)
    dC = dev(np.zeros((M, N), np.float32))
    gbblas.sgemm(ta, tb, M, N, K, 1.0, dev(A), A.shape[1], dev(B), B.shape[1], 0.0, dC, N,
                 algo=gbblas.ALGO_FP16X3)
    got = host(dC)
    a64, b64 = opA.astype(np.float64), opB.astype(np.float64)
    want = np.empty((M, N))
    with np.errstate(invalid="ignore", over="ignore"):
        for i in range(M):   # every product formed (a BLAS may skip zeros and lose Inf * 0 = NaN)
            want[i] = (a64[i][:, None] * b64).sum(axis=0)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert np.array_equal(np.isposinf(got), np.isposinf(want))
    assert np.array_equal(np.isneginf(got), np.isneginf(want))
    fin = np.isfinite(want)
    assert np.max(np.abs(got[fin] - want[fin])) <= 2 * K * 2.0 ** -24 * np.max(np.abs(want[fin]))


@pytest.mark.parametrize("chunk", ["0", "2", "16"])
def test_fp16x3_accumulation_chunks(torch, chunk):
    """Other accumulator chunks (0: one accumulator over all of K, no
    folding): exact on integers, within 2*K*u32 on U[-1,1]."""
    import os
    import gbblas
    os.environ["GB_FP16X3_FOLD"] = chunk
    try:
        M, N, K = 700, 520, 2000
        A, B = _ints(M, K, 25), _ints(K, N, 26)
        want = (A.astype(np.float64) @ B.astype(np.float64)).astype(np.float32)
        dC = dev(np.zeros((M, N), np.float32))
        gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=gbblas.ALGO_FP16X3)
        assert np.array_equal(host(dC), want)
        A = oracle.fill(M, K, 27, dtype=np.float32)
        B = oracle.fill(N, K, 28, dtype=np.float32)
        dC = dev(np.zeros((M, N), np.float32))
        gbblas.sgemm("N", "T", M, N, K, 1.0, dev(A), K, dev(B), K, 0.0, dC, N, algo=gbblas.ALGO_FP16X3)
        err, _ = oracle.normwise_error(host(dC), "N", "T", M, N, K, 1.0, A, K, B, K, 0.0, None, N,
                                       np.arange(0, M, 7), np.arange(0, N, 7))
        assert err <= 2 * K * 2.0 ** -24, err
    finally:
        os.environ.pop("GB_FP16X3_FOLD", None)


def test_bf16x3_folded_wide_form_exact(torch):
    """BF16X3 through the folding form with eight epilogue warps
    (GB_BF16X3_FOLD): exact on integers in all four modes."""
    import os
    import gbblas
    os.environ["GB_BF16X3_FOLD"] = "4"
    try:
        for mode in MODES:
            ta, tb = mode
            M, N, K = 1030, 700, 600
            ar, ac = op_shape(ta, M, K)
            br, bc = op_shape(tb, K, N)
            A, B, C0 = _ints(ar, ac, 31), _ints(br, bc, 32), _ints(M, N, 33)
            opA = A.T if ta == "T" else A
            opB = B.T if tb == "T" else B
            want = (opA.astype(np.float64) @ opB.astype(np.float64) - 0.5 * C0).astype(np.float32)
            dC = dev(C0)
            gbblas.sgemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, -0.5, dC, N, algo=gbblas.ALGO_BF16X3)
            assert np.array_equal(host(dC), want), mode
    finally:
        os.environ.pop("GB_BF16X3_FOLD", None)


@pytest.mark.parametrize("algo_name", ["BF16X3", "FP16X3"])
def test_two_pass_captured_in_cuda_graph(torch, algo_name):
    """A call captured into a CUDA graph (workspace reserved first) replays
    to the same bits as the eager call, also with eager calls of other shapes
    on the same stream between the replays."""
    import gbblas
    algo = getattr(gbblas, "ALGO_" + algo_name)
    tc = torch
    s = tc.cuda.Stream()
    M, N, K = 1024, 768, 1536
    A = dev(oracle.fill(M, K, 960, dtype=np.float32))
    B = dev(oracle.fill(K, N, 961, dtype=np.float32))
    A2 = dev(oracle.fill(512, 640, 962, dtype=np.float32))
    B2 = dev(oracle.fill(640, 384, 963, dtype=np.float32))
    assert gbblas.lib().gb_workspace_reserve(256 << 20, s.cuda_stream) == gbblas.OK
    C_ref = tc.zeros((M, N), dtype=tc.float32, device="cuda:0")
    C2_ref = tc.zeros((512, 384), dtype=tc.float32, device="cuda:0")
    with tc.cuda.stream(s):
        gbblas.sgemm("N", "N", M, N, K, 1.0, A, K, B, N, 0.0, C_ref, N, algo=algo, stream=s)
        gbblas.sgemm("N", "N", 512, 384, 640, 1.0, A2, 640, B2, 384, 0.0, C2_ref, 384, algo=algo, stream=s)
    s.synchronize()
    C = tc.zeros_like(C_ref)
    g = tc.cuda.CUDAGraph()
    with tc.cuda.graph(g, stream=s):
        gbblas.sgemm("N", "N", M, N, K, 1.0, A, K, B, N, 0.0, C, N, algo=algo, stream=s)
    C2 = tc.zeros_like(C2_ref)
    with tc.cuda.stream(s):
        for _ in range(3):
            C.zero_()
            g.replay()
            gbblas.sgemm("N", "N", 512, 384, 640, 1.0, A2, 640, B2, 384, 0.0, C2, 384, algo=algo, stream=s)
    s.synchronize()
    assert tc.equal(C, C_ref)
    assert tc.equal(C2, C2_ref)
