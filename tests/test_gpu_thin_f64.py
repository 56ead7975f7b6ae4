"""FP64 skinny products (thinB / shortA, n <= 64) through integer digits on
the tensor cores, against the oracle.

* Small-integer inputs: every digit product and every level sum is an exact
  integer, so the result must equal the exact product bit for bit -- this
  pins the FP64 tensor-map boxes, the digit slices in tensor memory, the 36
  digit pairs into 8 level accumulators, the column passes of 16 and the
  split-K parts.
* U[-1,1] and wide-exponent (u * 2^e, e in [-20, 20]) inputs: normwise error
  against the Dot2 oracle within 2*K*u64, and against the native FP64
  kernels (GB_SKINNY_OZ=0) within the same bound.
"""
import os

import numpy as np
import pytest

import oracle
from gpu_util import dev, host, op_shape, torch_cuda

pytestmark = pytest.mark.gpu
MODES = ["NN", "NT", "TN", "TT"]


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


def _ints(rows, cols, seed, ld):
    rng = np.random.default_rng(seed)
    X = np.zeros((rows, ld), dtype=np.float64)
    X[:, :cols] = rng.integers(-40, 41, size=(rows, cols)).astype(np.float64)
    return X


def _ld(c):
    return max(2, (c + 1) // 2 * 2)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("small,big,K", [(8, 3001, 1037), (16, 700, 96), (5, 1000, 640), (33, 257, 4099),
                                         (64, 2000, 600), (12, 60, 9000)])
@pytest.mark.parametrize("sem", [0, 2])
def test_thin_f64_exact_on_integers(torch, mode, kind, small, big, K, sem):
    import gbblas
    ta, tb = mode
    M, N = (big, small) if kind == "thinB" else (small, big)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    lda, ldb, ldc = _ld(ac), _ld(bc), N + 1
    A, B = _ints(ar, ac, 1, lda), _ints(br, bc, 2, ldb)
    C0 = _ints(M, N, 3, ldc)
    opA = A[:, :ac].T if ta == "T" else A[:, :ac]
    opB = B[:, :bc].T if tb == "T" else B[:, :bc]
    prod = opA @ opB        # integers below 2^53: exact in FP64
    want = C0.copy()
    if sem == 0:
        want[:, :N] = -1.0 * prod + 2.0 * C0[:, :N]
    else:
        want[:, :N] = C0[:, :N] + (-1.0 * prod + 2.0)
    dC = dev(C0)
    gbblas.dgemm(ta, tb, M, N, K, -1.0, dev(A), lda, dev(B), ldb, 2.0, dC, ldc, algo=gbblas.ALGO_SKINNY,
                 semantics=sem)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, kind, bad[:5])


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("small,fill", [(8, 0), (24, 2), (64, 0)])
def test_thin_f64_normwise_and_matches_native(torch, mode, kind, small, fill):
    import gbblas
    ta, tb = mode
    big, K = 4000, 2049
    M, N = (big, small) if kind == "thinB" else (small, big)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    lda, ldb, ldc = _ld(ac), _ld(bc), N
    A = oracle.fill(ar, ac, 81, kind=fill, dtype=np.float64, ld=lda)
    B = oracle.fill(br, bc, 82, kind=fill, dtype=np.float64, ld=ldb)
    C0 = oracle.fill(M, N, 83, kind=fill, dtype=np.float64, ld=ldc)
    outs = []
    for oz in ("1", "0"):
        os.environ["GB_SKINNY_OZ"] = oz
        try:
            dC = dev(C0)
            gbblas.dgemm(ta, tb, M, N, K, 0.75, dev(A), lda, dev(B), ldb, -0.5, dC, ldc, algo=gbblas.ALGO_SKINNY)
            outs.append(host(dC))
        finally:
            os.environ.pop("GB_SKINNY_OZ", None)
    rows = np.arange(0, M, max(1, M // 53))
    cols = np.arange(0, N, max(1, N // 53))
    for got in outs:
        err, _ = oracle.normwise_error(got, ta, tb, M, N, K, 0.75, A, lda, B, ldb, -0.5, C0, ldc, rows, cols)
        assert err <= 2 * K * 2.0 ** -53, err


def test_thin_f64_deterministic(torch):
    import gbblas
    M, N, K = 3000, 20, 20000
    A = oracle.fill(M, K, 91, dtype=np.float64)
    B = oracle.fill(K, N, 92, dtype=np.float64)
    outs = []
    for _ in range(2):
        dC = dev(np.zeros((M, N), np.float64))
        gbblas.dgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
        outs.append(host(dC))
    assert outs[0].tobytes() == outs[1].tobytes()


@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("xscale,wscale", [(-1000, 0), (-1060, 500), (600, -700)])
def test_thin_f64_exact_on_scaled_integers(torch, kind, xscale, wscale):
    """Small integers times 2^xscale (tiny and subnormal rows take the general
    mantissa path, normal rows the fast one; one warp mixes both) and W times
    2^wscale: the products stay exact, so the result must be bit-exact."""
    import gbblas
    big, small, K = 1000, 16, 700
    M, N = (big, small) if kind == "thinB" else (small, big)
    A = _ints(M, K, 5, K)
    B = _ints(K, N, 6, N)
    # the large operand gets the scale on every other row / column of 32
    if kind == "thinB":
        A[::2] *= 2.0 ** xscale
        B *= 2.0 ** wscale
    else:
        B[:, ::2] *= 2.0 ** xscale
        A *= 2.0 ** wscale
    want = A @ B
    dC = dev(np.zeros((M, N), np.float64))
    gbblas.dgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (kind, bad[:5], got[tuple(bad[0])] if bad.size else None)


def _check_nonfinite(got, want):
    assert np.array_equal(np.isnan(got), np.isnan(want))
    inf = np.isinf(want)
    assert np.array_equal(np.isinf(got), inf)
    assert np.array_equal(np.sign(got[inf]), np.sign(want[inf]))
    fin = np.isfinite(want)
    scale = np.abs(want[fin]).max()
    assert np.abs(got[fin] - want[fin]).max() <= 1e-12 * scale


@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("mode", ["NN", "TT"])
def test_thin_f64_nonfinite_propagate(torch, kind, mode):
    """An Inf or a NaN in the large operand's line or in a column of the
    small one reaches exactly the outputs that IEEE arithmetic gives it."""
    import gbblas
    ta, tb = mode
    big, small, K = 900, 24, 513
    M, N = (big, small) if kind == "thinB" else (small, big)
    rng = np.random.default_rng(7)
    opA = rng.uniform(-1, 1, (M, K))
    opB = rng.uniform(-1, 1, (K, N))
    opA[M // 3, 17] = np.inf
    opA[M - 1, K - 1] = np.nan
    opB[5, N // 2] = -np.inf
    opB[K // 2, 0] = np.nan
    opA[M // 2, 3] = opA[M // 2, 4] = np.inf      # Inf + (-Inf) -> NaN in one output
    opB[3, N - 1], opB[4, N - 1] = 1.0, -1.0
    A = np.ascontiguousarray(opA.T if ta == "T" else opA)
    B = np.ascontiguousarray(opB.T if tb == "T" else opB)
    want = opA @ opB
    dC = dev(np.zeros((M, N), np.float64))
    gbblas.dgemm(ta, tb, M, N, K, 1.0, dev(A), A.shape[1], dev(B), B.shape[1], 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
    _check_nonfinite(host(dC), want)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("small,big,K", [(8, 3001, 1037), (40, 1001, 777)])
def test_thin_f64_odd_ld_exact(torch, mode, kind, small, big, K):
    """Leading dimensions TMA cannot describe (odd, and a base 8 bytes off a
    16-byte boundary): the large operand is copied by cp.async; still exact."""
    import gbblas
    ta, tb = mode
    M, N = (big, small) if kind == "thinB" else (small, big)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    lda, ldb = ac | 1, bc | 1
    A, B = _ints(ar, ac, 11, lda), _ints(br, bc, 12, ldb)
    opA = A[:, :ac].T if ta == "T" else A[:, :ac]
    opB = B[:, :bc].T if tb == "T" else B[:, :bc]
    want = opA @ opB
    for offset in (0, 1):   # offset 1: the operand starts 8 bytes into the buffer
        dA = dev(np.concatenate([np.zeros(offset), A.ravel()]))
        dB = dev(np.concatenate([np.zeros(offset), B.ravel()]))
        dC = dev(np.zeros((M, N)))
        gbblas.dgemm(ta, tb, M, N, K, 1.0, dA[offset:], lda, dB[offset:], ldb, 0.0, dC, N,
                     algo=gbblas.ALGO_SKINNY)
        got = host(dC)
        bad = np.argwhere(got != want)
        assert bad.size == 0, (mode, kind, offset, bad[:5])


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
def test_thin_f64_cpasync_loader_matches_tma(torch, mode, kind):
    """The cp.async loader (forced on an aligned operand) fills shared memory
    exactly as the TMA boxes do: bit-identical results."""
    import gbblas
    ta, tb = mode
    big, small, K = 3000, 24, 1500
    M, N = (big, small) if kind == "thinB" else (small, big)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, 31, dtype=np.float64)
    B = oracle.fill(br, bc, 32, dtype=np.float64)
    outs = []
    for force in ("0", "1"):
        os.environ["GB_SKINNY_OZ_CPASYNC"] = force
        try:
            dC = dev(np.zeros((M, N)))
            gbblas.dgemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
            outs.append(host(dC))
        finally:
            os.environ.pop("GB_SKINNY_OZ_CPASYNC", None)
    assert outs[0].tobytes() == outs[1].tobytes()


@pytest.mark.parametrize("kind", ["thinB", "shortA"])
def test_thin_f64_split_k_nonfinite_and_odd_ld(torch, kind):
    """Few rows, long K: the digit kernel splits K (partials summed by the
    reduce kernel, Inf/NaN rows flagged per split); n = 40 takes a pass of
    two 16-column groups and one of one group; odd leading dimensions take the
    cp.async loader.  Finite outputs within 2*K*u normwise; Inf/NaN where
    numpy's product has them."""
    import gbblas
    small, big, K = 40, 300, 8192
    M, N = (big, small) if kind == "thinB" else (small, big)
    rng = np.random.default_rng(17)
    opA = rng.uniform(-1, 1, (M, K))
    opB = rng.uniform(-1, 1, (K, N))
    # one non-finite value in the large operand's line (row of A for thinB, column of B for shortA)
    if kind == "thinB":
        opA[7, 5000] = np.inf
        opA[M - 2, 100] = np.nan
    else:
        opB[5000, 7] = -np.inf
        opB[100, N - 2] = np.nan
    lda, ldb = K | 1, N | 1
    A = np.zeros((M, lda)); A[:, :K] = opA
    B = np.zeros((K, ldb)); B[:, :N] = opB
    want = opA @ opB
    dC = dev(np.zeros((M, N)))
    gbblas.dgemm("N", "N", M, N, K, 1.0, dev(A), lda, dev(B), ldb, 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
    got = host(dC)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    inf = np.isinf(want)
    assert np.array_equal(np.isinf(got), inf)
    assert np.array_equal(np.sign(got[inf]), np.sign(want[inf]))
    fin = np.isfinite(want)
    num = np.linalg.norm(got[fin] - want[fin])
    den = np.linalg.norm(np.abs(opA[np.isfinite(opA).all(1)]), "fro") * np.linalg.norm(opB[:, np.isfinite(opB).all(0)], "fro")
    assert num <= 2 * K * 2.0 ** -53 * den, num / den


@pytest.mark.parametrize("small", [8, 24])
def test_thin_f64_slow_epilogues_keep_chunk_exponents(torch, small):
    """Three row tiles per CTA, eight 256-k chunks each, and an Inf in one row
    of every tile: each tile's epilogue recomputes that row as a plain dot
    product (slow), while the converters run ahead into the next tile.  The
    exponents of every chunk must still reach the drain: finite outputs within
    2*K*u normwise, the Inf rows as numpy has them."""
    import gbblas
    M, N, K = 152 * 128 * 3, small, 2048
    rng = np.random.default_rng(23)
    A = rng.uniform(-1, 1, (M, K))
    A *= np.ldexp(1.0, rng.integers(-30, 30, size=(M, 1)))   # row scales differ
    B = rng.uniform(-1, 1, (K, N))
    A[5::128, 77] = np.inf
    want = A @ B
    dC = dev(np.zeros((M, N)))
    gbblas.dgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
    got = host(dC)
    inf_rows = np.zeros(M, bool)
    inf_rows[5::128] = True
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert np.array_equal(np.isinf(got), np.isinf(want))
    fin = ~inf_rows
    # per-row normwise error (rows have their own scales)
    num = np.linalg.norm(got[fin] - want[fin], axis=1)
    den = np.linalg.norm(A[fin], axis=1) * np.linalg.norm(B)
    assert np.all(num <= 2 * K * 2.0 ** -53 * den), (num / den).max()
