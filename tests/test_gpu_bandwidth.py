"""Transpose and Jacobi on the GPU against the oracle and the golden
fixtures: bit-exact."""
import hashlib

import numpy as np
import pytest

import gbgen
import golden_cases as gc
import oracle
from gpu_util import dev, host, torch_cuda

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.mark.parametrize("M,N", [(312, 228), (1512, 1536), (8210, 8190)])
def test_transpose_golden(torch, M, N):
    """transpose/bin/run.sh shapes; expected = the reference demo's B_ref."""
    import gbblas
    meta = gc.index()["transpose_f32_%dx%d" % (M, N)]
    dA = dev(gbgen.demo_transpose(M, N))
    dB = torch.zeros((N, M), dtype=torch.float32, device="cuda:0")
    gbblas.exec_by_name("transpose_float_32x32_dbuf", [M, N, 0], [dA, dB])
    assert hashlib.sha256(host(dB).tobytes()).hexdigest() == meta["sha256"]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("M,N,pa,pb", [(1, 1, 0, 0), (63, 65, 0, 0), (130, 257, 3, 5), (1000, 7, 1, 0),
                                         (7, 3000, 0, 2)])
def test_transpose_ld_bit_exact(torch, dtype, M, N, pa, pb):
    import gbblas
    A = oracle.fill(M, N, 77, dtype=dtype, ld=N + pa)
    A[:, N:] = np.nan                      # padding must not leak
    want = np.zeros((N, M + pb), dtype=dtype)
    oracle.transpose_into(M, N, A, N + pa, want, M + pb)
    dB = dev(np.zeros((N, M + pb), dtype=dtype))
    gbblas.transpose(M, N, dev(A), N + pa, dB, M + pb, 64 if dtype == np.float64 else 32)
    assert host(dB).tobytes() == want.tobytes()


def test_transpose_preserves_special_values(torch):
    import gbblas
    A = np.array([[-0.0, np.inf], [np.nan, -np.inf], [1e-320, 5.0]], dtype=np.float64)
    dB = dev(np.zeros((2, 3)))
    gbblas.transpose(3, 2, dev(A), 2, dB, 3, 64)
    assert host(dB).tobytes() == np.ascontiguousarray(A.T).tobytes()


@pytest.mark.parametrize("M,N", [(55, 111), (256, 300)])
def test_stencil_golden_one_sweep(torch, M, N):
    """one sweep in the host order equals the reference's reference_stencil."""
    import gbblas
    meta = gc.index()["stencil_f64_%dx%d" % (M, N)]
    A = gbgen.demo_stencil(M, N)
    dA, dB = dev(A), dev(np.zeros_like(A))
    gbblas.stencil2d(M, N, dA, dB, 1, gbblas.STENCIL_HOST, 64)
    got = np.ascontiguousarray(host(dB)[1:M + 1, 1:N + 1])
    assert hashlib.sha256(got.tobytes()).hexdigest() == meta["sha256"]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("M,N,iters", [(1, 1, 1), (33, 47, 2), (64, 130, 7), (200, 333, 17), (129, 64, 20),
                                      (300, 500, 30), (257, 1000, 16), (130, 113, 9)])
def test_stencil_iterations_bit_exact(torch, dtype, order, M, N, iters):
    import gbblas
    A = np.ones((M + 2, N + 2), dtype=dtype)            # Dirichlet boundary 1.0
    A[1:M + 1, 1:N + 1] = oracle.fill(M, N, 9, kind=1, dtype=dtype)
    B = A.copy()
    a, b = A.copy(), B.copy()
    oracle.stencil(M, N, a, b, iters, order)
    dA, dB = dev(A), dev(B)
    gbblas.stencil2d(M, N, dA, dB, iters, order, 64 if dtype == np.float64 else 32)
    res, want = (host(dB), b) if iters % 2 else (host(dA), a)
    assert res.tobytes() == want.tobytes()
    # the other buffer is scratch (it holds an earlier sweep); its halo is never written
    other = host(dA) if iters % 2 else host(dB)
    for edge in (np.s_[0, :], np.s_[-1, :], np.s_[:, 0], np.s_[:, -1]):
        assert other[edge].tobytes() == A[edge].tobytes()


def test_stencil_vector_entry_point(torch):
    import gbblas
    M, N = 40, 60
    A = gbgen.demo_stencil(M, N)
    a, b = A.copy(), np.zeros_like(A)
    oracle.stencil(M, N, a, b, 1, 2)
    dA, dB = dev(A), dev(np.zeros_like(A))
    assert gbblas.ref_call("stencil_vector", M, N, dA, dB) == gbblas.OK
    assert host(dB).tobytes() == b.tobytes()


def test_fill_matches_oracle(torch):
    import gbblas
    for bits, dt in ((64, np.float64), (32, np.float32)):
        for kind in (0, 1, 2):
            want = oracle.fill(123, 77, 99, kind=kind, dtype=dt, ld=80)
            d = dev(np.zeros_like(want))
            gbblas.fill(d, 123, 77, 80, 99, kind, bits)
            got = host(d)
            assert got[:, :77].tobytes() == np.ascontiguousarray(want[:, :77]).tobytes()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("M,N,pad", [(1, 1, 0), (63, 65, 3), (300, 129, 0), (1000, 777, 5)])
def test_transpose_add_bit_exact(torch, dtype, M, N, pad):
    """B += A^T, the reference's *_add transpose-accumulate, one IEEE add per element."""
    import gbblas
    bits = 64 if dtype == np.float64 else 32
    A = oracle.fill(M, N, 61, dtype=dtype, ld=N + pad)
    B = oracle.fill(N, M, 62, kind=2, dtype=dtype, ld=M + pad)
    want = B.copy()
    oracle.transpose_add_into(M, N, A, N + pad, want, M + pad)
    dB = dev(B)
    gbblas.transpose_add(M, N, dev(A), N + pad, dB, M + pad, bits)
    assert host(dB).tobytes() == want.tobytes()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("M,N,iters", [(1, 1, 1), (33, 47, 2), (200, 333, 9), (300, 500, 13), (257, 1000, 4),
                                      (130, 113, 7)])
def test_stencil9_bit_exact(torch, dtype, M, N, iters):
    """9-point stencil, arbitrary 3x3 weights: bit-identical to the
    product-then-eight-fmas recurrence, several sweeps per pass."""
    import gbblas
    rng = np.random.default_rng(M * 7 + N)
    w = rng.uniform(-0.3, 0.4, size=9).astype(dtype)
    A = np.ones((M + 2, N + 2), dtype=dtype)
    A[1:M + 1, 1:N + 1] = oracle.fill(M, N, 19, kind=1, dtype=dtype)
    B = A.copy()
    a, b = A.copy(), B.copy()
    oracle.stencil9(M, N, a, b, iters, w)
    dA, dB = dev(A), dev(B)
    gbblas.stencil9(M, N, dA, dB, iters, w, 64 if dtype == np.float64 else 32)
    res, want = (host(dB), b) if iters % 2 else (host(dA), a)
    assert res.tobytes() == want.tobytes()
    other = host(dA) if iters % 2 else host(dB)
    for edge in (np.s_[0, :], np.s_[-1, :], np.s_[:, 0], np.s_[:, -1]):
        assert other[edge].tobytes() == A[edge].tobytes()
