"""Per-call normwise error report (gb_gemm_opts.err_out).

The device estimate is compared with the oracle's normwise error on the same
sampled rows and columns (16 each, spread evenly: row i is
floor((2i+1) M / 32)): for BLAS semantics the two are the same measure (Dot2
reference rounded once to FP64), so they agree to rounding of the norms; for
the scalar-beta semantics the expected value is formed on the host from the
oracle's Dot2 product.  Every form of both precisions is covered, with
padded leading dimensions, M or N below the sample size, and M == 0.
"""
import numpy as np
import pytest

import oracle
from gpu_util import dev, host, op_shape, torch_cuda

pytestmark = pytest.mark.gpu

S = 16


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


def _sample(n):
    k = min(n, S)
    return np.array([((2 * i + 1) * n) // (2 * k) for i in range(k)], dtype=np.int64)


def _run(torch, bits, mode, M, N, K, algo, alpha, beta, sem, seed, pad=3):
    import gbblas
    dt = np.float64 if bits == 64 else np.float32
    ta, tb = mode
    ar, ac = op_shape(ta, M, K)
    br, bc = op_shape(tb, K, N)
    A = oracle.fill(ar, ac, seed, dtype=dt, ld=ac + pad)
    B = oracle.fill(br, bc, seed + 1, dtype=dt, ld=bc + pad)
    C0 = oracle.fill(M, N, seed + 2, dtype=dt, ld=N + pad)
    dA, dB, dC = dev(A), dev(B), dev(C0)
    err = torch.full((1,), -1.0, dtype=torch.float64, device="cuda:0")
    gbblas.gemm(ta, tb, M, N, K, alpha, dA, ac + pad, dB, bc + pad, beta, dC, N + pad, bits, algo=algo,
                semantics=sem, err_out=err)
    torch.cuda.synchronize()
    return A, ac + pad, B, bc + pad, C0, host(dC), float(err.item())


CASES = [
    (32, "NN", 300, 260, 500, "simt"), (32, "TN", 257, 129, 700, "bf16x3"), (32, "NT", 640, 512, 1000, "fp16x3"),
    (32, "TT", 384, 320, 640, "bf16x6"), (32, "NN", 70, 90, 300, "ordered"), (32, "NT", 5, 3000, 800, "skinny"),
    (64, "NN", 300, 260, 500, "ordered"), (64, "TN", 257, 300, 700, "dmma"), (64, "NT", 640, 512, 1000, "ozaki"),
    (64, "TT", 2500, 8, 900, "skinny"), (32, "NN", 12, 9, 40, "auto"),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s_f%d_%s_%dx%dx%d" % (c[5], c[0], c[1], c[2], c[3], c[4]))
def test_report_matches_oracle_normwise_error(torch, case):
    import gbblas
    bits, mode, M, N, K, name = case
    algo = {"auto": gbblas.ALGO_AUTO, "ordered": gbblas.ALGO_ORDERED, "simt": gbblas.ALGO_SIMT,
            "dmma": gbblas.ALGO_DMMA, "bf16x3": gbblas.ALGO_BF16X3, "bf16x6": gbblas.ALGO_BF16X6,
            "fp16x3": gbblas.ALGO_FP16X3, "ozaki": gbblas.ALGO_OZAKI, "skinny": gbblas.ALGO_SKINNY}[name]
    alpha, beta = 1.25, -0.75
    A, lda, B, ldb, C0, got, err = _run(torch, bits, mode, M, N, K, algo, alpha, beta, gbblas.SEM_BLAS, 41)
    want, _ = oracle.normwise_error(got, mode[0], mode[1], M, N, K, alpha, A, lda, B, ldb, beta, C0, C0.shape[1],
                                    _sample(M), _sample(N))
    assert err >= 0.0
    assert abs(err - want) <= 1e-9 * want + 1e-300, (err, want)
    u = 2.0 ** -53 if bits == 64 else 2.0 ** -24
    assert err <= 2 * K * u


@pytest.mark.parametrize("sem", [1, 2])
def test_report_scalar_beta_semantics(torch, sem):
    M, N, K, mode = 200, 150, 333, "NT"
    alpha, beta = 0.5, 2.0
    import gbblas
    A, lda, B, ldb, C0, got, err = _run(torch, 32, mode, M, N, K, gbblas.ALGO_SIMT, alpha, beta, sem, 77)
    rows, cols = _sample(M), _sample(N)
    prod = oracle.gemm_dot2(mode[0], mode[1], M, N, K, alpha, A, lda, B, ldb, 0.0, None, C0.shape[1], rows, cols)
    c0 = C0[np.ix_(rows, cols)].astype(np.float64)
    ref = prod + beta + (c0 if sem == gbblas.SEM_ACCUM_SCALAR_BETA else 0.0)
    rn2, cn2 = oracle.op_norms(mode[0], mode[1], M, N, K, A, lda, B, ldb, rows, cols)
    den = abs(alpha) * np.sqrt(rn2.sum() * cn2.sum()) + abs(beta) * np.sqrt(ref.size)
    if sem == gbblas.SEM_ACCUM_SCALAR_BETA:
        den += np.linalg.norm(c0)
    want = np.linalg.norm(got[np.ix_(rows, cols)].astype(np.float64) - ref) / den
    assert abs(err - want) <= 1e-6 * want, (err, want)
    assert err <= 2 * K * 2.0 ** -24


def test_report_empty_product_is_zero(torch):
    import gbblas
    err = torch.full((1,), -1.0, dtype=torch.float64, device="cuda:0")
    C = torch.zeros(4, dtype=torch.float32, device="cuda:0")
    gbblas.sgemm("N", "N", 0, 4, 8, 1.0, C, 8, C, 4, 0.0, C, 4, err_out=err)
    torch.cuda.synchronize()
    assert float(err.item()) == 0.0


@pytest.mark.parametrize("name", ["simt", "bf16x3", "fp16x3", "ozaki"])
def test_report_is_zero_for_exact_products(torch, name):
    """Small integers: every form computes the product exactly, so the
    reported error is exactly 0 (the report adds no error of its own)."""
    import gbblas
    bits = 64 if name == "ozaki" else 32
    dt = np.float64 if bits == 64 else np.float32
    algo = {"simt": gbblas.ALGO_SIMT, "bf16x3": gbblas.ALGO_BF16X3, "fp16x3": gbblas.ALGO_FP16X3,
            "ozaki": gbblas.ALGO_OZAKI}[name]
    M, N, K = 256, 192, 320
    rng = np.random.default_rng(9)
    A = rng.integers(-8, 9, size=(M, K)).astype(dt)
    B = rng.integers(-8, 9, size=(K, N)).astype(dt)
    C0 = rng.integers(-8, 9, size=(M, N)).astype(dt)
    dC = dev(C0)
    err = torch.full((1,), -1.0, dtype=torch.float64, device="cuda:0")
    gbblas.gemm("N", "N", M, N, K, 2.0, dev(A), K, dev(B), N, -1.0, dC, N, bits, algo=algo, err_out=err)
    torch.cuda.synchronize()
    assert float(err.item()) == 0.0
    want = 2.0 * (A.astype(np.float64) @ B.astype(np.float64)) - C0
    assert np.array_equal(host(dC).astype(np.float64), want)
