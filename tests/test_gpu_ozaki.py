"""Ozaki-slice DGEMM on tcgen05 against the oracle.

* Inputs whose rows/columns need few digits (small integers; values with a
  handful of significant bits spread over a wide exponent range): the slice
  representation is exact, every slice product is exact, and the result
  must equal the exact product (checked against Dot2 to the last bit where
  the exact result is representable).
* U[-1,1] and the precision-study distribution u*2^e, e in [-20, 20]
  (the DGEMM precision workload): normwise error against Dot2 falls
  with the slice count and at 7-8 slices is at FP64 level (<= 2*K*u64).
"""
import numpy as np
import pytest

import oracle
from gpu_util import dev, host, op_shape, torch_cuda

pytestmark = pytest.mark.gpu
MODES = ["NN", "NT", "TN", "TT"]


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


def _ints(rows, cols, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(-100, 101, size=(rows, cols)).astype(np.float64)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 300, 1100), (7, 9, 5), (300, 257, 2500)])
def test_ozaki_exact_on_integers(torch, mode, M, N, K):
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A, B, C0 = _ints(ar, ac, 1), _ints(br, bc, 2), _ints(M, N, 3)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    want = 2.0 * (opA @ opB) - 1.0 * C0          # exact: integers far below 2^53
    dC = dev(C0)
    gbblas.dgemm(ta, tb, M, N, K, 2.0, dev(A), ac, dev(B), bc, -1.0, dC, N, algo=gbblas.ALGO_OZAKI, ozaki_slices=2)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, bad[:5])


def test_ozaki_exact_products_on_wide_exponents(torch):
    """14 significant bits per entry, exponents spread over +-6 inside each row
    (at most 26 bits below the row maximum): every entry is at most 4 balanced
    base-256 digits (7 + 8 + 8 + 8 bits), so with 8 slices every digit
    product t + u <= 8 is kept and exact; only the FP64 summation of the 36
    scaled pair sums rounds."""
    import gbblas
    rng = np.random.default_rng(7)
    M, N, K = 160, 144, 700

    def make(r, c):
        m = rng.integers(-(2 ** 13), 2 ** 13, size=(r, c)).astype(np.float64)
        e = rng.integers(-6, 7, size=(r, c))
        return np.ldexp(m, e - 13)

    A, B = make(M, K), make(K, N)
    dC = dev(np.zeros((M, N)))
    gbblas.dgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=gbblas.ALGO_OZAKI, ozaki_slices=8)
    got = host(dC)
    ref = oracle.gemm_dot2("N", "N", M, N, K, 1.0, A, K, B, N, 0.0, None, N, np.arange(M), np.arange(N))
    scale = np.abs(A) @ np.abs(B)
    assert np.all(np.abs(got - ref) <= 2.0 ** -50 * scale)


@pytest.mark.parametrize("kind", [0, 2])
@pytest.mark.parametrize("mode", ["NN", "TT"])
def test_ozaki_error_falls_with_slices(torch, kind, mode):
    import gbblas
    ta, tb = mode
    M, N, K = 256, 384, 1024
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, 41, kind=kind)
    B = oracle.fill(br, bc, 42, kind=kind)
    C0 = oracle.fill(M, N, 43, kind=kind)
    rows, cols = np.arange(0, M, 3), np.arange(0, N, 3)
    errs = {}
    for s in (4, 5, 6, 7, 8, 9):
        dC = dev(C0)
        gbblas.dgemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, 1.0, dC, N, algo=gbblas.ALGO_OZAKI,
                     ozaki_slices=s)
        errs[s], _ = oracle.normwise_error(host(dC), ta, tb, M, N, K, 1.0, A, ac, B, bc, 1.0, C0, N, rows, cols)
    assert errs[8] <= 2 * K * 2.0 ** -53, errs
    assert errs[4] > errs[6] > errs[8] or errs[8] < 1e-15, errs
    # native FP64 (ordered DFMA) for comparison: Ozaki at 9 slices is no worse than it
    dC = dev(C0)
    gbblas.dgemm(ta, tb, M, N, K, 1.0, dev(A), ac, dev(B), bc, 1.0, dC, N, algo=gbblas.ALGO_ORDERED)
    native, _ = oracle.normwise_error(host(dC), ta, tb, M, N, K, 1.0, A, ac, B, bc, 1.0, C0, N, rows, cols)
    assert errs[8] <= 4 * native + 1e-17, (errs, native)
    assert errs[9] <= native, (errs, native)


@pytest.mark.parametrize("sem", [0, 1, 2])
def test_ozaki_semantics_and_auto_slices(torch, sem):
    import gbblas
    M, N, K = 130, 140, 300
    A, B, C0 = _ints(M, K, 4), _ints(K, N, 5), _ints(M, N, 6)
    exact = 0.5 * (A @ B)
    want = {0: exact + 2.0 * C0, 1: exact + 2.0, 2: C0 + (exact + 2.0)}[sem]
    dC = dev(C0)
    gbblas.dgemm("N", "N", M, N, K, 0.5, dev(A), K, dev(B), N, 2.0, dC, N, algo=gbblas.ALGO_OZAKI, semantics=sem)
    assert np.array_equal(host(dC), want)


def test_ozaki_zero_rows_and_columns(torch):
    import gbblas
    M, N, K = 100, 90, 200
    A, B = _ints(M, K, 8), _ints(K, N, 9)
    A[5, :] = 0.0
    B[:, 7] = 0.0
    dC = dev(np.zeros((M, N)))
    gbblas.dgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=gbblas.ALGO_OZAKI, ozaki_slices=3)
    assert np.array_equal(host(dC), A @ B)


def test_ozaki_k_chunked_matches_unchunked_error(torch):
    """K long enough that the slices are cut into K chunks (workspace cap):
    still FP64-level against Dot2."""
    import gbblas
    M, N, K = 640, 64, 400000          # 9 slices x (640 + 128) x K x 2 B > 4 GiB
    A = oracle.fill(M, K, 61)
    B = oracle.fill(K, N, 62)
    C0 = oracle.fill(M, N, 63)
    dC = dev(C0)
    gbblas.dgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, -1.0, dC, N, algo=gbblas.ALGO_OZAKI, ozaki_slices=9)
    rows, cols = np.arange(0, M, 20), np.arange(0, N, 4)
    err, _ = oracle.normwise_error(host(dC), "N", "N", M, N, K, 1.0, A, K, B, N, -1.0, C0, N, rows, cols)
    assert err <= 2 * K * 2.0 ** -53, err


@pytest.mark.parametrize("mode", ["NN", "TN", "NT", "TT"])
def test_ozaki_nonfinite_propagate(torch, mode):
    """Inf and NaN in a row of op(A) or a column of op(B) reach exactly the
    outputs that IEEE arithmetic gives them (those outputs are recomputed as
    plain dot products); the others keep FP64-level accuracy."""
    import gbblas
    ta, tb = mode
    M, N, K = 300, 260, 700
    rng = np.random.default_rng(11)
    opA = rng.uniform(-1, 1, (M, K))
    opB = rng.uniform(-1, 1, (K, N))
    opA[7, 100] = np.inf
    opA[M - 1, 0] = np.nan
    opB[9, 33] = -np.inf
    opB[K - 1, N - 1] = np.nan
    opA[150, 4] = opA[150, 5] = np.inf      # Inf + (-Inf) -> NaN in output (150, 200)
    opB[4, 200], opB[5, 200] = 1.0, -1.0
    A = np.ascontiguousarray(opA.T if ta == "T" else opA)
    B = np.ascontiguousarray(opB.T if tb == "T" else opB)
    want = opA @ opB
    dC = dev(np.zeros((M, N)))
    gbblas.dgemm(ta, tb, M, N, K, 1.0, dev(A), A.shape[1], dev(B), B.shape[1], 0.0, dC, N,
                 algo=gbblas.ALGO_OZAKI, ozaki_slices=7)
    got = host(dC)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    inf = np.isinf(want)
    assert np.array_equal(np.isinf(got), inf)
    assert np.array_equal(np.sign(got[inf]), np.sign(want[inf]))
    fin = np.isfinite(want)
    assert np.abs(got[fin] - want[fin]).max() <= 1e-12 * np.abs(want[fin]).max()


@pytest.mark.parametrize("mode", ["NN", "TN", "NT", "TT"])
@pytest.mark.parametrize("M,N,K", [(640, 768, 1100), (300, 513, 2100)])
def test_ozaki_wide_form_bit_identical_to_narrow(torch, mode, M, N, K):
    """The 128 x 256 form (N >= 256) does the 128 x 128 form's arithmetic in
    the same order: identical bits, ragged shapes and every layout, beta != 0
    and a K past one exact chunk (1024)."""
    import os
    import gbblas
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = dev(oracle.fill(ar, ac, 71, kind=2))
    B = dev(oracle.fill(br, bc, 72, kind=2))
    C0 = oracle.fill(M, N, 73)
    outs = []
    for wide in ("1", "0"):
        os.environ["GB_OZAKI_WIDE"] = wide
        try:
            C = dev(C0)
            gbblas.dgemm(ta, tb, M, N, K, 1.25, A, ac, B, bc, -0.5, C, N, algo=gbblas.ALGO_OZAKI)
            outs.append(host(C).tobytes())
        finally:
            os.environ.pop("GB_OZAKI_WIDE", None)
    assert outs[0] == outs[1]
