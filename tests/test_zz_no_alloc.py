"""gb_sgemm_skinny_noalloc: the skinny FP32 GEMM that allocates no device
memory, for callers that cannot allocate on the call path (a serving loop
working inside a fixed HBM budget, a framework whose device memory belongs to
its own pool allocator, code that must not hit cudaFree's implicit
synchronisation).

It is called through the C ABI and compared with the existing entry point
(gb_sgemm with GB_ALGO_SKINNY) on the same inputs, on two calls in a row whose
split-K plans use the shared scratch array: within the normwise 2*K*u32
tolerance the other GEMM tests use for 8 < min(M, N) <= 64 (there the
existing entry point runs on the tensor cores), and bit for bit for
min(M, N) <= 8 (the same kernels and plan), including the layouts whose small
operand is packed into the scratch array first.  A fresh process checks that
the first calls change the device's free memory by nothing.  This file is
named so pytest collects it last.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import oracle
from gpu_util import dev, host, op_shape, torch_cuda

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


# min(M, N) <= 8, split-K: (mode, M, N, K, extra lda, extra ldb).  The second
# case has a row-major large operand with ld % 4 != 0 and a small operand
# with an odd ld: the small operand is packed into the scratch array (at an
# offset past the partial sums) before the streaming kernel reads it; the
# third is the shortA mirror of that.
SMALL_CASES = [("NN", 3000, 8, 20000, 0, 0), ("NN", 2000, 5, 9001, 0, 2), ("NT", 7, 2500, 7001, 0, 0)]


@pytest.mark.parametrize("case", SMALL_CASES)
def test_noalloc_small_n_bit_identical_to_skinny_two_calls(torch, case):
    import gbblas
    L = gbblas.lib()
    mode, M, N, K, pa, pb = case
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, 110, dtype=np.float32, ld=ac + pa)
    B = oracle.fill(br, bc, 210, dtype=np.float32, ld=bc + pb)
    C0 = oracle.fill(M, N, 310, dtype=np.float32)
    dA, dB = dev(A), dev(B)
    c_ref = dev(C0)
    gbblas.sgemm(ta, tb, M, N, K, 1.25, dA, ac + pa, dB, bc + pb, 0.5, c_ref, N, algo=gbblas.ALGO_SKINNY)
    want = host(c_ref)
    for _ in range(2):   # two calls in a row, both through the shared scratch array
        c_new = dev(C0)
        st = _noalloc(L, ta, tb, M, N, K, 1.25, dA, ac + pa, dB, bc + pb, 0.5, c_new, N)
        assert st == gbblas.OK, L.gb_last_error()
        assert L.gb_sync(None) == gbblas.OK
        assert host(c_new).tobytes() == want.tobytes()


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


# Run in a fresh process with every module loaded when the context is made
# (CUDA_MODULE_LOADING=EAGER), so that nothing but an allocation can change
# the device's free memory: the first two calls of the process, on the
# min(M, N) <= 8 streaming path (split-K partials and a packed small operand
# in the scratch array), must leave it unchanged.
_FRESH = textwrap.dedent("""
    import ctypes, glob, sys
    sys.path.insert(0, %(pkg)r)
    import gbblas
    L = gbblas.lib()
    libs = sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
    libs += sorted(glob.glob("/usr/local/cuda/targets/*/lib/libcudart.so*"))
    if not libs:
        print("NO_CUDART")
        sys.exit(0)
    rt = ctypes.CDLL(libs[0])

    def free_bytes():
        f, t = ctypes.c_size_t(), ctypes.c_size_t()
        assert rt.cudaMemGetInfo(ctypes.byref(f), ctypes.byref(t)) == 0
        return f.value

    f = L.gb_sgemm_skinny_noalloc
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_float,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]
    f.restype = ctypes.c_int
    M, N, K, lda, ldb = 2000, 5, 9001, 9001, 7
    ptrs = []
    for nbytes in (M * lda * 4, K * ldb * 4, M * N * 4):
        p = ctypes.c_void_p()
        assert L.gb_malloc(ctypes.byref(p), nbytes) == 0
        ptrs.append(p.value)
    A, B, C = ptrs
    gbblas.fill(A, M, K, lda, 1, bits=32)
    gbblas.fill(B, K, N, ldb, 2, bits=32)
    assert L.gb_sync(None) == 0
    free0 = free_bytes()
    for _ in range(2):
        st = f(b"N", b"N", M, N, K, 1.0, A, lda, B, ldb, 0.0, C, N, 0, None)
        assert st == 0, L.gb_last_error()
    assert L.gb_sync(None) == 0
    free1 = free_bytes()
    print("FREE", free0, free1)
    assert free1 == free0, (free0, free1)
""")


def test_noalloc_first_calls_allocate_nothing_in_a_fresh_process(torch):
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    code = _FRESH % {"pkg": os.path.join(REPO, "blas-for-multi-core-dsp_gb300")}
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    if "NO_CUDART" in r.stdout:
        pytest.skip("no libcudart.so to read the device's free memory with")
    assert "FREE" in r.stdout
