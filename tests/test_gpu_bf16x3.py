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
