"""gb_sgemm_skinny_noalloc: the skinny FP32 GEMM that allocates no device
memory, for callers that cannot allocate on the call path (a serving loop
working inside a fixed HBM budget, a framework whose device memory belongs to
its own pool allocator, code that must not hit cudaFree's implicit
synchronisation).

It is called through the C ABI and compared with the existing entry point
(gb_sgemm with GB_ALGO_SKINNY) on the same inputs, within the normwise
2*K*u32 tolerance the other GEMM tests use, on two calls in a row whose
split-K plans use the shared scratch array.  This file is named so pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

import oracle
from gpu_util import dev, host, op_shape, torch_cuda

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


def _noalloc(L, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, semantics=0):
    f = L.gb_sgemm_skinny_noalloc
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_float,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f(ta.encode(), tb.encode(), M, N, K, alpha, A.data_ptr(), lda, B.data_ptr(), ldb, beta,
             C.data_ptr(), ldc, semantics, None)


# (mode, M, N, K): both use split-K (few rows, long K), so both go through the scratch array
CASES = [("NN", 1500, 16, 30000), ("TN", 12, 2000, 25000)]


def test_noalloc_matches_skinny_entry_point_two_calls(torch):
    import gbblas
    L = gbblas.lib()
    for i, (mode, M, N, K) in enumerate(CASES):
        ta, tb = mode
        ar, ac = op_shape(ta, M, K)
        br, bc = op_shape(tb, K, N)
        A = oracle.fill(ar, ac, 100 + i, dtype=np.float32)
        B = oracle.fill(br, bc, 200 + i, dtype=np.float32)
        C0 = oracle.fill(M, N, 300 + i, dtype=np.float32)
        dA, dB = dev(A), dev(B)
        c_ref, c_new = dev(C0), dev(C0)
        gbblas.sgemm(ta, tb, M, N, K, 0.75, dA, ac, dB, bc, -1.5, c_ref, N, algo=gbblas.ALGO_SKINNY)
        st = _noalloc(L, ta, tb, M, N, K, 0.75, dA, ac, dB, bc, -1.5, c_new, N)
        assert st == gbblas.OK, L.gb_last_error()
        assert L.gb_sync(None) == gbblas.OK
        ref, new = host(c_ref).astype(np.float64), host(c_new).astype(np.float64)
        rn2, cn2 = oracle.op_norms(ta, tb, M, N, K, A, ac, B, bc, np.arange(M), np.arange(N))
        den = 0.75 * np.sqrt(rn2.sum() * cn2.sum()) + 1.5 * np.linalg.norm(C0.astype(np.float64))
        assert np.linalg.norm(new - ref) / den <= 2 * K * 2.0 ** -24
        # and against the Dot2 oracle on a row/column sample
        rows = np.arange(0, M, max(1, M // 40))
        cols = np.arange(0, N, max(1, N // 40))
        err, _ = oracle.normwise_error(host(c_new), ta, tb, M, N, K, 0.75, A, ac, B, bc, -1.5, C0, N, rows, cols)
        assert err <= 2 * K * 2.0 ** -24


def test_noalloc_rejects_plans_beyond_the_fixed_scratch(torch):
    import gbblas
    L = gbblas.lib()
    # thinB with op(A) stored K x M (the K-major kernel, 256 rows per CTA):
    # 5000 rows make 20 row tiles, so the plan splits K 16 ways and needs
    # 16 x 5000 x 64 x 4 B = 20.5 MB of partials > 16 MiB.  The buffers are
    # full size, so the call is memory-safe even if a plan ever fits.
    M, N, K = 5000, 64, 4096
    A = torch.zeros((K, M), dtype=torch.float32, device="cuda:0")
    B = torch.zeros((K, N), dtype=torch.float32, device="cuda:0")
    C = torch.zeros((M, N), dtype=torch.float32, device="cuda:0")
    st = _noalloc(L, "T", "N", M, N, K, 1.0, A, M, B, N, 0.0, C, N)
    assert st == gbblas.ERR_INVALID_ARG
    assert b"16777216" in L.gb_last_error()
    assert L.gb_sync(None) == gbblas.OK
