"""The streamed FP32 skinny kernels against the oracle: the TMA/FFMA kernel
(n = min(M, N) <= 8) and the tensor-core kernel (8 < n <= 64, K >= 64, X
split into BF16 hi/lo in tensor memory), both for 16-byte aligned operands
with leading dimensions a multiple of 4.

* Small-integer inputs: every product and partial sum is an integer below
  2^24, so any summation order gives the exact result -- this pins the
  tensor-map boxes, the 128-byte swizzle of row-major X, both W layouts,
  zero fill beyond K / rows / n, the split-K partials and the strided
  C writes of the shortA (transposed) form.
* U[-1,1] inputs: normwise error against the Dot2 oracle <= 2*K*u32, and
  the same call with the streamed kernel switched off (GB_SKINNY_TMA=0)
  agrees to the same bound.
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
    X = np.zeros((rows, ld), dtype=np.float32)
    X[:, :cols] = rng.integers(-4, 5, size=(rows, cols)).astype(np.float32)
    return X


def _ld(c):
    return max(4, (c + 3) // 4 * 4)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("small,big,K", [(8, 3001, 1037), (1, 700, 96), (3, 1000, 33), (5, 257, 4099),
                                         (4, 60, 3000), (8, 513, 20000), (12, 3001, 1037), (16, 700, 96),
                                         (40, 1000, 640), (64, 257, 4099), (33, 60, 3000), (64, 2000, 64)])
@pytest.mark.parametrize("sem", [0, 1, 2])
def test_thin_exact_on_integers(torch, mode, kind, small, big, K, sem):
    import gbblas
    ta, tb = mode
    M, N = (big, small) if kind == "thinB" else (small, big)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    lda, ldb, ldc = _ld(ac), _ld(bc), N + 3
    A, B = _ints(ar, ac, 1, lda), _ints(br, bc, 2, ldb)
    C0 = _ints(M, N, 3, ldc)
    opA = A[:, :ac].T if ta == "T" else A[:, :ac]
    opB = B[:, :bc].T if tb == "T" else B[:, :bc]
    prod = opA.astype(np.float64) @ opB.astype(np.float64)
    assert np.abs(prod).max() < 2 ** 24
    want = C0.copy()
    if sem == 0:
        want[:, :N] = (-1.0 * prod + 2.0 * C0[:, :N]).astype(np.float32)
    elif sem == 1:
        want[:, :N] = (-1.0 * prod + 2.0).astype(np.float32)
    else:
        want[:, :N] = (C0[:, :N] + (-1.0 * prod + 2.0)).astype(np.float32)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, -1.0, dev(A), lda, dev(B), ldb, 2.0, dC, ldc, algo=gbblas.ALGO_SKINNY,
                 semantics=sem)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, kind, bad[:5])


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("small", [2, 8, 16, 64])
def test_thin_normwise_and_matches_unstreamed(torch, mode, kind, small):
    import gbblas
    ta, tb = mode
    big, K = 5000, 2049
    M, N = (big, small) if kind == "thinB" else (small, big)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    lda, ldb, ldc = _ld(ac), _ld(bc), N
    A = oracle.fill(ar, ac, 71, dtype=np.float32, ld=lda)
    B = oracle.fill(br, bc, 72, dtype=np.float32, ld=ldb)
    C0 = oracle.fill(M, N, 73, dtype=np.float32, ld=ldc)
    outs = []
    for on in ("1", "0"):
        os.environ["GB_SKINNY_TMA"] = os.environ["GB_SKINNY_TC"] = on
        try:
            dC = dev(C0)
            gbblas.sgemm(ta, tb, M, N, K, 0.5, dev(A), lda, dev(B), ldb, -1.0, dC, ldc, algo=gbblas.ALGO_SKINNY)
            outs.append(host(dC))
        finally:
            os.environ.pop("GB_SKINNY_TMA", None)
            os.environ.pop("GB_SKINNY_TC", None)
    rows = np.arange(0, M, max(1, M // 61))
    cols = np.arange(0, N, max(1, N // 61))
    for got in outs:
        err, _ = oracle.normwise_error(got, ta, tb, M, N, K, 0.5, A, lda, B, ldb, -1.0, C0, ldc, rows, cols)
        assert err <= 2 * K * 2.0 ** -24, err
    den = np.linalg.norm(outs[1].astype(np.float64)) + 1.0
    assert np.linalg.norm(outs[0].astype(np.float64) - outs[1]) / den <= 2 * K * 2.0 ** -24


def test_thin_deterministic(torch):
    """Fixed K split and k-ordered FMAs: two runs give identical bits."""
    import gbblas
    M, N, K = 2000, 8, 30000
    A = oracle.fill(M, K, 81, dtype=np.float32)
    B = oracle.fill(K, N, 82, dtype=np.float32)
    outs = []
    for _ in range(2):
        dC = dev(np.zeros((M, N), np.float32))
        gbblas.sgemm("N", "N", M, N, K, 1.0, dev(A), K, dev(B), N, 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
        outs.append(host(dC))
    assert outs[0].tobytes() == outs[1].tobytes()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["thinB", "shortA"])
@pytest.mark.parametrize("small,big,K,mis", [(12, 3001, 1037, 1), (33, 1000, 640, 2), (64, 2000, 4099, 3),
                                             (16, 700, 96, 1), (40, 60, 3000, 3), (8, 900, 513, 1),
                                             (3, 1001, 2050, 2), (8, 40, 9000, 3)])
def test_thin_unaligned_leading_dimension_exact(torch, mode, kind, small, big, K, mis):
    """Leading dimensions that are not a multiple of 4 floats: row-major X is
    streamed as four row classes with phase-shifted W pieces (tensor-core
    form); the other layouts take the register-streaming kernels.  Integer
    inputs: exact in any order."""
    import gbblas
    ta, tb = mode
    M, N = (big, small) if kind == "thinB" else (small, big)
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    lda, ldb, ldc = ac + mis, bc + mis, N + mis
    A, B = _ints(ar, ac, 21, lda), _ints(br, bc, 22, ldb)
    C0 = _ints(M, N, 23, ldc)
    opA = A[:, :ac].T if ta == "T" else A[:, :ac]
    opB = B[:, :bc].T if tb == "T" else B[:, :bc]
    want = C0.copy()
    want[:, :N] = (0.5 * (opA.astype(np.float64) @ opB.astype(np.float64)) - 3.0 * C0[:, :N]).astype(np.float32)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 0.5, dev(A), lda, dev(B), ldb, -3.0, dC, ldc, algo=gbblas.ALGO_SKINNY)
    got = host(dC)
    bad = np.argwhere(got != want)
    assert bad.size == 0, (mode, kind, bad[:5])


@pytest.mark.parametrize("mode", ["NN", "NT", "TN", "TT"])
@pytest.mark.parametrize("N", [8, 24])
def test_thin_unaligned_nan_in_previous_row_does_not_leak(torch, mode, N):
    """The class decomposition reads a few values before each row start (the
    previous row's tail); they are zeroed before use, so a NaN there must not
    reach the result."""
    import gbblas
    ta, tb = mode
    M, K = 2000, 515                 # thinB; lda = K + 1 when A is row-major
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    lda, ldb = ac + 1, bc
    A = oracle.fill(ar, ac, 91, dtype=np.float32, ld=lda)
    A[:, ac:] = np.nan               # padding between rows
    B = oracle.fill(br, bc, 92, dtype=np.float32, ld=ldb)
    C0 = np.zeros((M, N), np.float32)
    dC = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 1.0, dev(A), lda, dev(B), ldb, 0.0, dC, N, algo=gbblas.ALGO_SKINNY)
    got = host(dC)
    assert np.isfinite(got).all()
    rows = np.arange(0, M, 37)
    err, _ = oracle.normwise_error(got, ta, tb, M, N, K, 1.0, A, lda, B, ldb, 0.0, C0, N, rows, np.arange(N))
    assert err <= 2 * K * 2.0 ** -24, err
