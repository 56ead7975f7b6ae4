"""gb_workspace_query against the calls it sizes.

The queried bytes, reserved on a fresh stream, carry the call captured into
a CUDA graph on that stream: the library's workspace refuses to grow while
a capture is open, so a bound that is too small fails the capture.  The
replay must equal the eager call bit for bit.
"""
import numpy as np
import pytest

import oracle
from gpu_util import dev, torch_cuda

pytestmark = pytest.mark.gpu

# (bits, algorithm, modes, M, N, K): split-operand forms, Ozaki slices, skinny split-K parts
CASES = [(32, "FP16X3", "NN", 1024, 768, 1536), (32, "BF16X6", "TN", 512, 640, 1024),
         (64, "OZAKI", "NT", 768, 512, 1024), (32, "SKINNY", "NN", 20000, 16, 3000),
         (64, "SKINNY", "TN", 20000, 16, 3000), (64, "SKINNY", "NN", 12, 30000, 2000)]


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.mark.parametrize("bits,algo_name,mode,M,N,K", CASES)
def test_queried_workspace_carries_a_captured_call(torch, bits, algo_name, mode, M, N, K):
    import gbblas
    tc = torch
    algo = getattr(gbblas, "ALGO_" + algo_name)
    dt = np.float64 if bits == 64 else np.float32
    ta, tb = mode
    ar, ac = (K, M) if ta == "T" else (M, K)
    br, bc = (N, K) if tb == "T" else (K, N)
    A = dev(oracle.fill(ar, ac, 970, dtype=dt))
    B = dev(oracle.fill(br, bc, 971, dtype=dt))
    C0 = dev(oracle.fill(M, N, 972, dtype=dt))
    # the eager call on a stream of its own (it also does the per-device setup outside any capture)
    s1 = tc.cuda.Stream()
    C_ref = C0.clone()
    tc.cuda.synchronize()
    with tc.cuda.stream(s1):
        gbblas.gemm(ta, tb, M, N, K, 1.0, A, ac, B, bc, 0.5, C_ref, N, bits, algo=algo, stream=s1)
    s1.synchronize()
    # a fresh stream with only the queried bytes reserved, the same call captured there
    s2 = tc.cuda.Stream()
    nbytes = gbblas.workspace_query(bits, ta, tb, M, N, K, ac, bc, A=A, B=B, algo=algo)
    assert nbytes > 0
    gbblas.workspace_reserve(nbytes, s2)
    C = C0.clone()
    tc.cuda.synchronize()
    g = tc.cuda.CUDAGraph()
    with tc.cuda.graph(g, stream=s2, capture_error_mode="thread_local"):
        gbblas.gemm(ta, tb, M, N, K, 1.0, A, ac, B, bc, 0.5, C, N, bits, algo=algo, stream=s2)
    with tc.cuda.stream(s2):
        g.replay()
    s2.synchronize()
    assert tc.equal(C, C_ref)
