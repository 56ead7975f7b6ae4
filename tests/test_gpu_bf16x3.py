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
@pytest.mark.parametrize("M,N,K", [(4096, 4096, 320), (2048, 4096, 96), (4000, 3900, 1000)])
def test_bf16x3_stream_k_tail_exact(torch, mode, M, N, K):
    """Tile counts that leave a partial last wave, with the stream-K tail
    switched on (GB_BF16X3_SK=1): the tail tiles are split in K over two CTAs
    and summed by the second finisher.  Small integers keep every partial sum
    exact, so the result must equal the exact product."""
    import os
    import gbblas
    os.environ["GB_BF16X3_SK"] = "1"
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A, B = _ints(ar, ac, 31), _ints(br, bc, 32)
    C0 = _ints(M, N, 33)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    want = (opA.astype(np.float64) @ opB.astype(np.float64) - 2.0 * C0).astype(np.float32)
    try:
        for _ in range(2):   # twice: the part counters must be back at zero
            dC = dev(C0)
            gbblas.sgemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, -2.0, dC, N, algo=gbblas.ALGO_BF16X3)
            got = host(dC)
            bad = np.argwhere(got != want)
            assert bad.size == 0, (mode, bad[:5])
    finally:
        os.environ.pop("GB_BF16X3_SK", None)


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
